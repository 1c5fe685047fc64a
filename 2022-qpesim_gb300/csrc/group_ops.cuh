// group_ops.cuh - term application by a group of warps with every amplitude
// update split over four lanes.
//
// On GB300 a warp's FP64 instruction occupies its SM sub-partition's FP64 unit
// for many cycles, so a term applied by one warp costs (FP64 instructions per
// lane) x that issue time however many other warps are idle. Here a tile is
// processed by a group of warps (one per sub-partition) and each pair update of
// updateStateVector (cpp/time_evolution_over_terms.hpp:565-589) is done by a
// quad of lanes: lane q of the quad computes one real component of the result
// (l'.re, l'.im, r'.re, r'.im). Every component is the same expression, in the
// same operation order, as in pair_update (tile_ops.cuh), written as
//   out = x1*c1 + x2*c2                 (m00 real, m01 imaginary: 3 FP64 ops)
//   out = (x1*c1 + x2*c2) + (x3*c3 + x4*c4)   (general 2 x 2 matrix)
// with a subtraction written as the addition of the exactly negated product,
// so the result is bit-identical to the reference's complex arithmetic. Lanes
// pick their operands by q, so the quad runs one instruction stream.
//
// Within one term the pairs are disjoint; the quad reads both amplitudes of its
// pair before any lane writes (a warp barrier between the two), and a group
// barrier separates consecutive terms.
#ifndef QPE_GROUP_OPS_CUH_
#define QPE_GROUP_OPS_CUH_

#include "tile_ops.cuh"

namespace qpe {

// One term after another on a tile of W lines. left(w, e) / right(w, e) are the
// amplitudes a pair entry (e01, e10) of line w pairs up (the same accessor for
// a COL or ROW line; the b01 and b10 columns of column pair w in a MIX tile);
// diagonal terms use left. lstr(w) is line w's occupation string (for the
// terms' conditions), nvalid the number of real lines (< W at the block's
// edge), parb(w) the beta-pair parity of MIX column pair w (0 otherwise; MIX
// terms carry no conditions). gt is the thread's index in the group, gthreads
// the group size, gbar() the group barrier.
template <typename R, class A, bool G, class Left, class Right, class Lstr, class Parb, class Bar>
__device__ __forceinline__ void group_ops(const DevOp* __restrict__ ops, const double* __restrict__ coef,
                                          const uint32_t* __restrict__ pool, uint32_t op0, uint32_t op1, bool rev,
                                          uint32_t L, uint32_t logW, uint32_t nvalid, bool mix, uint32_t gt,
                                          uint32_t gthreads, Left left, Right right, Lstr lstr, Parb parb, Bar gbar) {
  using C2 = typename Cx<R>::T;
  const uint32_t n = op1 - op0;
  if (n == 0) return;
  const uint32_t q = gt & 3u, slot = gt >> 2, nslots = gthreads >> 2;
  // Items are (line w, entry j) with item = j * W + w; the slots step by
  // nslots (a multiple of W), so a thread's line w is fixed for the tile and
  // its line constants are loaded once.
  const uint32_t w = slot & ((1u << logW) - 1);
  const uint32_t j0 = slot >> logW, jstep = nslots >> logW;
  const uint32_t jshift = __ffs(jstep) - 1;  // jstep is a power of two
  const bool wvalid = w < nvalid;
  const uint32_t my_lstr = (!mix && wvalid) ? lstr(w) : 0u;
  const uint32_t my_parb = (mix && wvalid) ? parb(w) : 0u;
  // Operand and result components of quad lane q for a pair (l, r) whose m00
  // is real (c) and m01 imaginary (+-t), in R units from the amplitude start:
  //   q0: l'.x = l.x c - r.y t    q1: l'.y = l.y c + r.x t
  //   q2: r'.x = r.x c - l.y t    q3: r'.y = l.x t + r.y c
  const bool x1_from_r = q == 2, x2_from_r = q != 2;
  const uint32_t x1_comp = q == 1 ? 1u : 0u, x2_comp = q == 1 ? 0u : 1u;
  const bool dst_r = q >= 2;
  const uint32_t dst_comp = q & 1u;
  for (uint32_t i = 0; i < n; ++i) {
    const OpR<R> op = load_op<R, G>(ops, coef, rev ? op1 - 1 - i : op0 + i);
    const DevOp& d = op.d;
    const Coef4<R>& k = op.k;
    const uint32_t per_line = d.kind == OPK_DIAG_ALL ? L : d.count;
    const bool line_on = wvalid && (mix || d.ncond == 0 || cond_ok(my_lstr, d));
    // this lane's coefficients for either parity (reduced pair) or the diagonal
    R c1e, c1o, c2e, c2o;
    if (d.kind == OPK_PAIR) {
      const R c = k.e0r, te = k.e1i, to = k.o1i;  // m01 = i t, t = te (parity 0) or to (parity 1)
      c1e = q == 3 ? te : c;
      c1o = q == 3 ? to : c;
      c2e = q == 3 ? c : ((q & 1) ? te : neg(te));
      c2o = q == 3 ? c : ((q & 1) ? to : neg(to));
    } else {
      c1e = c1o = q ? k.e0i : k.e0r;
      c2e = c2o = q ? k.e0r : neg(k.e0i);
    }
    uint2 x = (d.kind == OPK_PAIR && j0 < per_line) ? ldm<G>(reinterpret_cast<const uint2*>(pool + d.tab) + j0)
                                                    : make_uint2(0u, 0u);
    // the same trip count for every thread of the group (the warp barrier below)
    const uint32_t ntrips = (per_line + jstep - 1) >> jshift;
    for (uint32_t t = 0; t < ntrips; ++t) {
      const uint32_t j = j0 + t * jstep;
      const bool act = line_on && j < per_line;
      uint2 xn = make_uint2(0u, 0u);
      if (d.kind == OPK_PAIR && j + jstep < per_line)
        xn = ldm<G>(reinterpret_cast<const uint2*>(pool + d.tab) + j + jstep);
      R out = (R)0;
      R* dst = nullptr;
      if (act) {
        if (d.kind == OPK_PAIR) {
          R* lp = reinterpret_cast<R*>(&left(w, x.x & 0x7fffffffu));
          R* rp = reinterpret_cast<R*>(&right(w, x.y));
          const uint32_t par = (x.x >> 31) ^ my_parb;
          if (k.reduced) {
            const R x1 = (x1_from_r ? rp : lp)[x1_comp];
            const R x2 = (x2_from_r ? rp : lp)[x2_comp];
            out = A::add(A::mul(x1, par ? c1o : c1e), A::mul(x2, par ? c2o : c2e));
          } else {
            // l' = l m00 + r m01, r' = l m01 + r m00, every complex product (ac - bd, ad + bc)
            const C2 vl = *reinterpret_cast<const C2*>(lp), vr = *reinterpret_cast<const C2*>(rp);
            const R m0r = par ? k.o0r : k.e0r, m0i = par ? k.o0i : k.e0i;
            const R m1r = par ? k.o1r : k.e1r, m1i = par ? k.o1i : k.e1i;
            const R ma_r = q < 2 ? m0r : m1r, ma_i = q < 2 ? m0i : m1i;  // multiplies l
            const R mb_r = q < 2 ? m1r : m0r, mb_i = q < 2 ? m1i : m0i;  // multiplies r
            const bool im = q & 1;
            const R g1 = im ? ma_i : ma_r, g2 = im ? ma_r : neg(ma_i);
            const R g3 = im ? mb_i : mb_r, g4 = im ? mb_r : neg(mb_i);
            out = A::add(A::add(A::mul(vl.x, g1), A::mul(vl.y, g2)), A::add(A::mul(vr.x, g3), A::mul(vr.y, g4)));
          }
          dst = (dst_r ? rp : lp) + dst_comp;
        } else if (q < 2) {
          const uint32_t e = d.kind == OPK_DIAG_LIST ? ldm<G>(pool + d.tab + j) : j;
          R* vp = reinterpret_cast<R*>(&left(w, e));
          // (vx c.r - vy c.i, vx c.i + vy c.r)
          out = A::add(A::mul(vp[0], c1e), A::mul(vp[1], c2e));
          dst = vp + q;
        }
      }
      __syncwarp();
      if (dst) *dst = out;
      x = xn;
    }
    gbar();
  }
}

// The terms of a column-pair (MIX) pass on a group tile of W column pairs: the
// lean form of group_ops for the inline pair matrices every term of the
// reference's getters has (m00 = c for both parities, m01 = i t for parity 0
// and -i t for parity 1). With t_p the parity's t, the four results of a pair
// (l, r) are
//   q0: l'.x = l.x c + r.y (-t_p)   q1: l'.y = l.y c + r.x t_p
//   q2: r'.x = r.x c + l.y (-t_p)   q3: r'.y = r.y c + l.x t_p
// which are updateStateVector's (cpp/time_evolution_over_terms.hpp:565-589)
// expressions bit for bit: a - b*t is a + b*(-t) exactly, and the sum of two
// products does not depend on their order. So lane q reads component x1 (the
// one it writes) and x2, and does two multiplications and one addition; x2 is
// the x1 of quad lane q ^ 3, so it comes by a shuffle and no lane reads an
// element another lane writes.
//
// A term is a chain through shared memory (load, three FP64 operations, store,
// group barrier), so everything else is taken off that chain: terms go in
// chunks of kMixChunk whose descriptors, table entries, coefficients and element
// addresses are all loaded and computed before the chunk's first update. Lanes
// without a pair in a warp that has some work on `scratch` (a group-private
// element) instead of branching; a warp with no pair in a term skips it.
// Passes with a term of more entries than the group has quads, or with a
// general matrix (a coefficient record), take the term-by-term loop below.
constexpr uint32_t kMixChunk = 4;

template <typename R, class A, bool G, class Left, class Right, class Parb, class Bar>
__device__ __forceinline__ void group_mix_ops(const DevOp* __restrict__ ops, const double* __restrict__ coef,
                                              const uint32_t* __restrict__ pool, uint32_t op0, uint32_t op1,
                                              bool rev, uint32_t logW, uint32_t nvalid, uint32_t gt,
                                              uint32_t gthreads, Left left, Right right, Parb parb, Bar gbar,
                                              typename Cx<R>::T* scratch) {
  using C2 = typename Cx<R>::T;
  const uint32_t n = op1 - op0;
  if (n == 0) return;
  const uint32_t q = gt & 3u, slot = gt >> 2, nslots = gthreads >> 2;
  const uint32_t w = slot & ((1u << logW) - 1);
  const uint32_t j0 = slot >> logW, jstep = nslots >> logW;
  const uint32_t wj0 = ((gt & ~31u) >> 2) >> logW;  // smallest j0 of this thread's warp
  const bool wvalid = w < nvalid;
  const uint32_t my_parb = wvalid ? parb(w) : 0u;
  const bool side1 = q >= 2;                  // x1 (and the result) on the right amplitude
  const uint32_t comp1 = q & 1u, comp2 = comp1 ^ 1u;
  const uint32_t sflip = comp1 ^ 1u;          // q0, q2 multiply x2 by -t_p
  auto desc = [&](uint32_t i, uint4& a, uint4& b) {
    const uint4* src = reinterpret_cast<const uint4*>(ops + (rev ? op1 - 1 - i : op0 + i));
    a = ldm<G>(src);
    b = ldm<G>(src + 1);
  };
  // entry j of a table of `count` entries (clamped: lanes past the end read the last one)
  auto entry = [&](uint32_t tab, uint32_t count, uint32_t j) {
    return count ? ldm<G>(reinterpret_cast<const uint2*>(pool + tab) + min(j, count - 1)) : make_uint2(0u, 0u);
  };
  // Fast path: every term inline with at most jstep entries (one trip).
  bool fast = true;
  for (uint32_t i = 0; i < n && fast; ++i) {
    const uint4 d = ldm<G>(reinterpret_cast<const uint4*>(ops + op0 + i));
    fast = d.w == OP_INLINE && d.y <= jstep;
  }
  if (fast) {
    for (uint32_t i0 = 0; i0 < n; i0 += kMixChunk) {
      R cc[kMixChunk], ss[kMixChunk];
      R* dp[kMixChunk];
      bool wact[kMixChunk];
#pragma unroll
      for (uint32_t k = 0; k < kMixChunk; ++k) {
        cc[k] = ss[k] = (R)0;
        dp[k] = reinterpret_cast<R*>(scratch);
        wact[k] = false;
        if (i0 + k < n) {
          uint4 a, b;
          desc(i0 + k, a, b);
          const uint2 x = entry(a.x, a.y, j0);
          const bool act = wvalid && j0 < a.y;
          wact[k] = wj0 < a.y;
          cc[k] = (R)__hiloint2double((int)b.y, (int)b.x);
          const R t = (R)__hiloint2double((int)b.w, (int)b.z);
          ss[k] = (((x.x >> 31) ^ my_parb ^ sflip) && act) ? neg(t) : t;
          if (act) {
            R* lp = reinterpret_cast<R*>(&left(w, x.x & 0x7fffffffu));
            R* rp = reinterpret_cast<R*>(&right(w, x.y));
            dp[k] = (side1 ? rp : lp) + comp1;
          } else {
            dp[k] = reinterpret_cast<R*>(scratch) + comp1;
          }
        }
      }
#pragma unroll
      for (uint32_t k = 0; k < kMixChunk; ++k) {
        if (i0 + k < n) {
          if (wact[k]) {
            const R x1 = *dp[k];
            const R x2 = __shfl_xor_sync(0xffffffffu, x1, 3);
            *dp[k] = A::add(A::mul(x1, cc[k]), A::mul(x2, ss[k]));
          }
          gbar();
        }
      }
    }
    return;
  }
  uint4 a, b;  // DevOp words: a = (tab, count, kind | ncond | cb0 | cb1, gen), b = (c0, c1)
  desc(0, a, b);
  uint2 x = entry(a.x, a.y, j0);
  for (uint32_t i = 0; i < n; ++i) {
    uint4 na, nb;
    desc(min(i + 1, n - 1), na, nb);
    const uint2 nx = entry(na.x, na.y, j0);
    const uint32_t tab = a.x, count = a.y;
    const uint32_t ntrips = (count + jstep - 1) / jstep;
    if (a.w == OP_INLINE) {
      const R c = (R)__hiloint2double((int)b.y, (int)b.x), t = (R)__hiloint2double((int)b.w, (int)b.z);
      const R tn = neg(t);
      for (uint32_t tr = 0; tr < ntrips; ++tr) {
        const uint32_t j = j0 + tr * jstep;
        const uint2 xn = entry(tab, count, j + jstep);
        if (wj0 + tr * jstep < count) {  // some lane of the warp has a pair
          const bool act = wvalid && j < count;
          R* lp = act ? reinterpret_cast<R*>(&left(w, x.x & 0x7fffffffu)) : reinterpret_cast<R*>(scratch);
          R* rp = act ? reinterpret_cast<R*>(&right(w, x.y)) : reinterpret_cast<R*>(scratch);
          const uint32_t par = (x.x >> 31) ^ my_parb;
          R* dst = (side1 ? rp : lp) + comp1;
          const R x1 = *dst, x2 = (side1 ? lp : rp)[comp2];
          const R out = A::add(A::mul(x1, c), A::mul(x2, (par ^ sflip) ? tn : t));
          __syncwarp();
          *dst = out;
        }
        x = xn;
      }
    } else {
      // general matrix: l' = l m00 + r m01, r' = l m01 + r m00 (group_ops' general update)
      const double2* cr = reinterpret_cast<const double2*>(coef + 8 * (size_t)a.w);
      const double2 e0 = __ldg(cr), e1 = __ldg(cr + 1), o0 = __ldg(cr + 2), o1 = __ldg(cr + 3);
      for (uint32_t tr = 0; tr < ntrips; ++tr) {
        const uint32_t j = j0 + tr * jstep;
        const uint2 xn = entry(tab, count, j + jstep);
        R out = (R)0;
        R* dst = nullptr;
        if (wvalid && j < count) {
          R* lp = reinterpret_cast<R*>(&left(w, x.x & 0x7fffffffu));
          R* rp = reinterpret_cast<R*>(&right(w, x.y));
          const uint32_t par = (x.x >> 31) ^ my_parb;
          const C2 vl = *reinterpret_cast<const C2*>(lp), vr = *reinterpret_cast<const C2*>(rp);
          const R m0r = (R)(par ? o0.x : e0.x), m0i = (R)(par ? o0.y : e0.y);
          const R m1r = (R)(par ? o1.x : e1.x), m1i = (R)(par ? o1.y : e1.y);
          const R ma_r = q < 2 ? m0r : m1r, ma_i = q < 2 ? m0i : m1i;  // multiplies l
          const R mb_r = q < 2 ? m1r : m0r, mb_i = q < 2 ? m1i : m0i;  // multiplies r
          const bool im = q & 1;
          const R g1 = im ? ma_i : ma_r, g2 = im ? ma_r : neg(ma_i);
          const R g3 = im ? mb_i : mb_r, g4 = im ? mb_r : neg(mb_i);
          out = A::add(A::add(A::mul(vl.x, g1), A::mul(vl.y, g2)), A::add(A::mul(vr.x, g3), A::mul(vr.y, g4)));
          dst = (q >= 2 ? rp : lp) + (q & 1);
        }
        __syncwarp();
        if (dst) *dst = out;
        x = xn;
      }
    }
    gbar();
    a = na;
    b = nb;
    x = nx;
  }
}


// The terms of a row or column pass on one line (a tile of W = 1) by a group,
// in the form of group_mix_ops: a pair update split over a quad (lane q writes
// component q of the pair, the partner component from lane q ^ 3), a diagonal
// update over a lane pair. For a diagonal coefficient (c0, c1) the two results
// of cmul (tile_ops.cuh: v.x c0 - v.y c1, v.x c1 + v.y c0) are
//   h0: v.x c0 + v.y (-c1)      h1: v.y c0 + v.x c1
// bit for bit, so lane h reads its own component, takes the other from lane
// h ^ 1 and does two multiplications and one addition, like a quad lane.
//
// A term whose conditions (occupied orbitals of the line's own string) fail is
// skipped by the whole group: the tile is one line. Terms with one update per
// lane (at most gthreads / 4 pairs or gthreads / 2 diagonal entries) and an
// inline matrix are set up kLineChunk at a time ahead of their updates; a term
// with more entries runs its trips one after another, and a general pair matrix
// takes group_ops' general quad update.
constexpr uint32_t kLineChunk = 4;

template <typename R, class A, bool G, class Elem, class Bar>
__device__ __forceinline__ void group_line_ops(const DevOp* __restrict__ ops, const double* __restrict__ coef,
                                               const uint32_t* __restrict__ pool, uint32_t op0, uint32_t op1,
                                               bool rev, uint32_t L, uint32_t lstr, uint32_t gt, uint32_t gthreads,
                                               Elem elem, Bar gbar, typename Cx<R>::T* scratch) {
  using C2 = typename Cx<R>::T;
  const uint32_t n = op1 - op0;
  if (n == 0) return;
  const uint32_t q = gt & 3u, pslot = gt >> 2, pstep = gthreads >> 2;  // pair updates: quads
  const uint32_t h = gt & 1u, dslot = gt >> 1, dstep = gthreads >> 1;  // diagonal updates: lane pairs
  const uint32_t wp0 = (gt & ~31u) >> 2, wd0 = (gt & ~31u) >> 1;       // this warp's smallest slots
  const bool side1 = q >= 2;
  const uint32_t comp1 = q & 1u, sflip = comp1 ^ 1u;
  R* const scr = reinterpret_cast<R*>(scratch);
  auto desc = [&](uint32_t i, uint4& a, uint4& b) {
    const uint4* src = reinterpret_cast<const uint4*>(ops + (rev ? op1 - 1 - i : op0 + i));
    a = ldm<G>(src);
    b = ldm<G>(src + 1);
  };
  auto cond = [&](uint32_t z) {  // z = kind | ncond << 8 | cb0 << 16 | cb1 << 24
    const uint32_t nc = (z >> 8) & 0xffu;
    uint32_t m = 0;
    if (nc > 0) m |= 1u << ((z >> 16) & 0xffu);
    if (nc > 1) m |= 1u << (z >> 24);
    return (lstr & m) == m;
  };
  // One update item of this lane: its own component, the coefficient pair and
  // the shuffle distance to the lane holding the other operand.
  struct Item {
    R* dp;
    R c, s;
    uint32_t xd;
    bool wact;
  };
  // Item of trip `tr` of an inline term (a, b) with `count` entries.
  auto make_item = [&](const uint4& a, const uint4& b, uint32_t count, uint32_t tr) {
    Item it;
    const uint32_t kind = a.z & 0xffu;
    it.c = (R)__hiloint2double((int)b.y, (int)b.x);
    const R c1 = (R)__hiloint2double((int)b.w, (int)b.z);
    if (kind == OPK_PAIR) {
      const uint32_t j = pslot + tr * pstep;
      const bool act = j < count;
      const uint2 x = ldm<G>(reinterpret_cast<const uint2*>(pool + a.x) + min(j, count - 1));
      it.s = (((x.x >> 31) ^ sflip) && act) ? neg(c1) : c1;
      R* lp = reinterpret_cast<R*>(&elem(x.x & 0x7fffffffu));
      R* rp = reinterpret_cast<R*>(&elem(x.y));
      it.dp = act ? (side1 ? rp : lp) + comp1 : scr + comp1;
      it.xd = 3;
      it.wact = wp0 + tr * pstep < count;
    } else {
      const uint32_t j = dslot + tr * dstep;
      const bool act = j < count;
      const uint32_t e = kind == OPK_DIAG_LIST ? ldm<G>(pool + a.x + min(j, count - 1)) : min(j, count - 1);
      it.s = h ? c1 : neg(c1);
      it.dp = act ? reinterpret_cast<R*>(&elem(e)) + h : scr + h;
      it.xd = 1;
      it.wact = wd0 + tr * dstep < count;
    }
    return it;
  };
  auto run_item = [&](const Item& it) {
    if (it.wact) {
      const R x1 = *it.dp;
      const R x2 = __shfl_xor_sync(0xffffffffu, x1, it.xd);
      *it.dp = A::add(A::mul(x1, it.c), A::mul(x2, it.s));
    }
  };
  uint32_t i = 0;
  while (i < n) {
    // Set up the next run of up to kLineChunk terms that are skipped or have one
    // inline update per lane; stop before the first other term.
    // The chunk's first descriptor words are loaded together (indices clamped
    // to the pass), so that its setup waits on one shared-memory round trip
    // for them and one for the entries, not on one chain per term.
    Item its[kLineChunk];
    bool has[kLineChunk];
    uint32_t m = 0;
    bool stop = false;
    uint4 da[kLineChunk];
#pragma unroll
    for (uint32_t k = 0; k < kLineChunk; ++k) {
      const uint32_t ik = min(i + k, n - 1);
      da[k] = ldm<G>(reinterpret_cast<const uint4*>(ops + (rev ? op1 - 1 - ik : op0 + ik)));
    }
#pragma unroll
    for (uint32_t k = 0; k < kLineChunk; ++k) {
      has[k] = false;
      its[k] = Item{scr, (R)0, (R)0, 1u, false};
      if (!stop && i + k < n) {
        const uint4 a = da[k];
        const uint4 b = ldm<G>(reinterpret_cast<const uint4*>(ops + (rev ? op1 - 1 - (i + k) : op0 + (i + k))) + 1);
        const uint32_t kind = a.z & 0xffu;
        const uint32_t count = kind == OPK_DIAG_ALL ? L : a.y;
        if (!cond(a.z) || count == 0) {
          m = k + 1;  // skipped by the whole group: no update, no barrier
        } else if (a.w == OP_INLINE && count <= (kind == OPK_PAIR ? pstep : dstep)) {
          its[k] = make_item(a, b, count, 0);
          has[k] = true;
          m = k + 1;
        } else {
          stop = true;
        }
      }
    }
#pragma unroll
    for (uint32_t k = 0; k < kLineChunk; ++k) {
      if (has[k]) {
        run_item(its[k]);
        gbar();
      }
    }
    i += m;
    if (stop) {
      // term i: several trips, or a general pair matrix
      uint4 a, b;
      desc(i, a, b);
      const uint32_t kind = a.z & 0xffu;
      const uint32_t count = kind == OPK_DIAG_ALL ? L : a.y;
      if (a.w == OP_INLINE) {
        const uint32_t ntrips = (count + (kind == OPK_PAIR ? pstep : dstep) - 1) / (kind == OPK_PAIR ? pstep : dstep);
        for (uint32_t tr = 0; tr < ntrips; ++tr) run_item(make_item(a, b, count, tr));
      } else {
        const double2* cr = reinterpret_cast<const double2*>(coef + 8 * (size_t)a.w);
        const double2 e0 = __ldg(cr), e1 = __ldg(cr + 1), o0 = __ldg(cr + 2), o1 = __ldg(cr + 3);
        for (uint32_t j = pslot; j < count + (pstep - 1) - ((count + pstep - 1) % pstep); j += pstep) {
          R out = (R)0;
          R* dst = nullptr;
          if (j < count) {
            const uint2 x = ldm<G>(reinterpret_cast<const uint2*>(pool + a.x) + j);
            R* lp = reinterpret_cast<R*>(&elem(x.x & 0x7fffffffu));
            R* rp = reinterpret_cast<R*>(&elem(x.y));
            const uint32_t par = x.x >> 31;
            const C2 vl = *reinterpret_cast<const C2*>(lp), vr = *reinterpret_cast<const C2*>(rp);
            const R m0r = (R)(par ? o0.x : e0.x), m0i = (R)(par ? o0.y : e0.y);
            const R m1r = (R)(par ? o1.x : e1.x), m1i = (R)(par ? o1.y : e1.y);
            const R ma_r = q < 2 ? m0r : m1r, ma_i = q < 2 ? m0i : m1i;  // multiplies l
            const R mb_r = q < 2 ? m1r : m0r, mb_i = q < 2 ? m1i : m0i;  // multiplies r
            const bool im = q & 1;
            const R g1 = im ? ma_i : ma_r, g2 = im ? ma_r : neg(ma_i);
            const R g3 = im ? mb_i : mb_r, g4 = im ? mb_r : neg(mb_i);
            out = A::add(A::add(A::mul(vl.x, g1), A::mul(vl.y, g2)), A::add(A::mul(vr.x, g3), A::mul(vr.y, g4)));
            dst = (q >= 2 ? rp : lp) + (q & 1);
          }
          __syncwarp();
          if (dst) *dst = out;
        }
      }
      gbar();
      ++i;
    }
  }
}

}  // namespace qpe

#endif  // QPE_GROUP_OPS_CUH_
