// tile_ops.cuh - the per-tile term application shared by the evolution kernels.
//
// A tile is W lines of one pass (program.h). Lane l of the warp owns line
// l % W for the whole tile and walks the entries j = l / W, l / W + 32 / W, ... of
// every term's index table, so each lane keeps its line's constants (column,
// beta-pair columns, occupation string) in registers. The pair update is the
// reference's updateStateVector (cpp/time_evolution_over_terms.hpp:565-589):
// l' = l*m00 + r*m01, r' = l*m01 + r*m00. In exact mode every product and sum of
// the complex128 arithmetic is rounded separately, in the order of
// std::complex<double>'s (ac - bd, ad + bc), so results are bit-identical to the
// reference built without floating-point contraction; terms whose m00 is real and
// m01 imaginary (every pq / pqqr / pqrs term of the Hamiltonian getters) skip the
// products with exact zeros, which changes no bit.
#ifndef QPE_TILE_OPS_CUH_
#define QPE_TILE_OPS_CUH_

#include <cuda_runtime.h>
#include <stdint.h>

#include "program.h"

namespace qpe {

template <typename R>
struct Cx;
template <>
struct Cx<double> {
  using T = double2;
};
template <>
struct Cx<float> {
  using T = float2;
};

struct ExactD {
  static __device__ __forceinline__ double mul(double a, double b) { return __dmul_rn(a, b); }
  static __device__ __forceinline__ double add(double a, double b) { return __dadd_rn(a, b); }
  static __device__ __forceinline__ double sub(double a, double b) { return __dsub_rn(a, b); }
};
template <typename R>
struct Fast {
  static __device__ __forceinline__ R mul(R a, R b) { return a * b; }
  static __device__ __forceinline__ R add(R a, R b) { return a + b; }
  static __device__ __forceinline__ R sub(R a, R b) { return a - b; }
};

// Metadata load: through the read-only data cache when the program's tables and
// term descriptors are in global memory (G), a plain load when a kernel has
// staged them in shared memory.
template <bool G, class T>
__device__ __forceinline__ T ldm(const T* p) {
  if constexpr (G) return __ldg(p);
  else return *p;
}

// Exact negation as a sign-bit flip on the integer pipe. On this GPU an FP64
// instruction occupies a warp's FP64 unit for about 64 cycles, so a negation
// written as FP64 arithmetic would cost as much as a product.
__device__ __forceinline__ double neg(double x) {
  return __longlong_as_double(__double_as_longlong(x) ^ (long long)0x8000000000000000ull);
}
__device__ __forceinline__ float neg(float x) { return __int_as_float(__float_as_int(x) ^ (int)0x80000000u); }

template <typename R>
struct Coef4 {
  R e0r, e0i, e1r, e1i, o0r, o0i, o1r, o1i;
  bool reduced;  // m00 real and m01 imaginary for both parities
};

// A term's descriptor with its coefficients in registers.
template <typename R>
struct OpR {
  DevOp d;
  Coef4<R> k;
};

// icoef, when given, replaces the inline (c0, c1) of op o with icoef[o]: the
// instances of a batch share one program's structure and keep their own
// coefficients.
template <typename R, bool G = true>
__device__ __forceinline__ OpR<R> load_op(const DevOp* __restrict__ ops, const double* __restrict__ coef, uint32_t o,
                                          const double2* __restrict__ icoef = nullptr) {
  OpR<R> r;
  const uint4* src = reinterpret_cast<const uint4*>(ops + o);
  const uint4 a = ldm<G>(src), b = ldm<G>(src + 1);
  r.d.tab = a.x;
  r.d.count = a.y;
  r.d.kind = (uint8_t)(a.z & 0xff);
  r.d.ncond = (uint8_t)((a.z >> 8) & 0xff);
  r.d.cb0 = (uint8_t)((a.z >> 16) & 0xff);
  r.d.cb1 = (uint8_t)(a.z >> 24);
  r.d.gen = a.w;
  r.d.c0 = __hiloint2double((int)b.y, (int)b.x);
  r.d.c1 = __hiloint2double((int)b.w, (int)b.z);
  if (icoef) {
    const double2 c = __ldg(icoef + o);
    r.d.c0 = c.x;
    r.d.c1 = c.y;
  }
  if (r.d.gen == OP_INLINE) {
    // diagonal (c0, c1); pair m00 = c0, m01 = i c1 (parity 0) / -i c1 (parity 1)
    r.k.e0r = r.k.o0r = (R)r.d.c0;
    r.k.e0i = r.k.o0i = (R)0;
    r.k.e1r = r.k.o1r = (R)0;
    r.k.e1i = (R)r.d.c1;
    r.k.o1i = neg((R)r.d.c1);
    r.k.reduced = r.d.kind == OPK_PAIR;
    if (r.d.kind != OPK_PAIR) r.k.e0i = (R)r.d.c1;
  } else {
    const double2* c = reinterpret_cast<const double2*>(coef + 8 * (size_t)r.d.gen);
    const double2 x0 = __ldg(c), x1 = __ldg(c + 1), x2 = __ldg(c + 2), x3 = __ldg(c + 3);
    r.k.e0r = (R)x0.x; r.k.e0i = (R)x0.y; r.k.e1r = (R)x1.x; r.k.e1i = (R)x1.y;
    r.k.o0r = (R)x2.x; r.k.o0i = (R)x2.y; r.k.o1r = (R)x3.x; r.k.o1i = (R)x3.y;
    r.k.reduced = false;
  }
  return r;
}

template <class A, typename R>
__device__ __forceinline__ void cmul(R ar, R ai, R br, R bi, R& outr, R& outi) {
  outr = A::sub(A::mul(ar, br), A::mul(ai, bi));
  outi = A::add(A::mul(ar, bi), A::mul(ai, br));
}

template <class A, typename C2, typename R>
__device__ __forceinline__ void pair_update(C2& l, C2& r, const Coef4<R>& k, uint32_t par) {
  const R m0r = par ? k.o0r : k.e0r, m0i = par ? k.o0i : k.e0i;
  const R m1r = par ? k.o1r : k.e1r, m1i = par ? k.o1i : k.e1i;
  const C2 vl = l, vr = r;
  C2 nl, nr;
  if (k.reduced) {
    // m00 = (c, 0), m01 = (0, t): l' = (lx c - ry t, ly c + rx t), r' = (rx c - ly t, lx t + ry c).
    nl.x = A::sub(A::mul(vl.x, m0r), A::mul(vr.y, m1i));
    nl.y = A::add(A::mul(vl.y, m0r), A::mul(vr.x, m1i));
    nr.x = A::sub(A::mul(vr.x, m0r), A::mul(vl.y, m1i));
    nr.y = A::add(A::mul(vl.x, m1i), A::mul(vr.y, m0r));
  } else {
    R ar, ai, br, bi;
    cmul<A>(vl.x, vl.y, m0r, m0i, ar, ai);
    cmul<A>(vr.x, vr.y, m1r, m1i, br, bi);
    nl.x = A::add(ar, br);
    nl.y = A::add(ai, bi);
    cmul<A>(vl.x, vl.y, m1r, m1i, ar, ai);
    cmul<A>(vr.x, vr.y, m0r, m0i, br, bi);
    nr.x = A::add(ar, br);
    nr.y = A::add(ai, bi);
  }
  l = nl;
  r = nr;
}

template <class A, typename C2, typename R>
__device__ __forceinline__ void diag_update(C2& v, const Coef4<R>& k) {
  R xr, xi;
  cmul<A>(v.x, v.y, k.e0r, k.e0i, xr, xi);
  v.x = xr;
  v.y = xi;
}

// The barrier between consecutive terms of a tile: the warp's, or the CTA's when
// a whole CTA shares one tile.
struct WarpSync {
  __device__ __forceinline__ void operator()() const { __syncwarp(); }
};
struct CtaSync {
  __device__ __forceinline__ void operator()() const { __syncthreads(); }
};

__device__ __forceinline__ bool cond_ok(uint32_t line_str, const DevOp& op) {
  uint32_t m = 0;
  if (op.ncond > 0) m |= 1u << op.cb0;
  if (op.ncond > 1) m |= 1u << op.cb1;
  return (line_str & m) == m;
}

// Runs the terms [op0, op1) of a COL or ROW pass on this lane's line, in order,
// or in reverse order when `rev` (the backward half of a second-order step).
// `elem(e)` returns a reference to entry e of the line; `active` is false for
// lanes past the last line; `lstr` is the line's occupation string (for
// conditions). The loop is software-pipelined: the next term's descriptor,
// coefficients and this lane's first table entry are loaded while the current
// term computes, so the chain of dependent terms pays shared-memory latency
// rather than the latency of the metadata loads.
template <typename R, class A, bool G = true, class Elem, class Sync = WarpSync>
__device__ __forceinline__ void run_line_ops(const DevOp* __restrict__ ops, const double* __restrict__ coef,
                                             const uint32_t* __restrict__ pool, uint32_t op0, uint32_t op1, bool rev,
                                             uint32_t L, uint32_t jl, uint32_t jstep, bool active, uint32_t lstr,
                                             Elem elem, const double2* __restrict__ icoef = nullptr,
                                             Sync sync = Sync()) {
  const uint32_t n = op1 - op0;
  if (n == 0) return;
  auto at = [&](uint32_t i) { return rev ? op1 - 1 - i : op0 + i; };
  auto first_of = [&](const DevOp& d) -> uint2 {
    return (d.kind == OPK_PAIR && jl < d.count) ? ldm<G>(reinterpret_cast<const uint2*>(pool + d.tab) + jl)
                                                : make_uint2(0u, 0u);
  };
  OpR<R> op = load_op<R, G>(ops, coef, at(0), icoef);
  uint2 first = first_of(op.d);
  for (uint32_t i = 0; i < n; ++i) {
    OpR<R> opn = op;
    uint2 firstn = make_uint2(0u, 0u);
    if (i + 1 < n) {
      opn = load_op<R, G>(ops, coef, at(i + 1), icoef);
      firstn = first_of(opn.d);
    }
    const DevOp& d = op.d;
    if (active && (d.ncond == 0 || cond_ok(lstr, d))) {
      if (d.kind == OPK_PAIR) {
        const uint2* __restrict__ t = reinterpret_cast<const uint2*>(pool + d.tab);
        uint2 x = first;
        for (uint32_t j = jl; j < d.count; j += jstep) {
          const uint32_t jn = j + jstep;
          const uint2 xn = jn < d.count ? ldm<G>(t + jn) : make_uint2(0u, 0u);
          pair_update<A>(elem(x.x & 0x7fffffffu), elem(x.y), op.k, x.x >> 31);
          x = xn;
        }
      } else if (d.kind == OPK_DIAG_LIST) {
        for (uint32_t j = jl; j < d.count; j += jstep) diag_update<A>(elem(ldm<G>(pool + d.tab + j)), op.k);
      } else {
        for (uint32_t e = jl; e < L; e += jstep) diag_update<A>(elem(e), op.k);
      }
    }
    sync();
    op = opn;
    first = firstn;
  }
}

// Runs the pqrs ABBA terms [op0, op1) of a MIX pass on this lane's column pair
// (reverse order when `rev`): entry (a01 | par, a10) pairs left(a01) with
// right(a10), parity adding the beta pair's parity parb
// (cpp/time_evolution_over_terms.hpp:774). Pipelined as run_line_ops.
template <typename R, class A, bool G = true, class Left, class Right, class Sync = WarpSync>
__device__ __forceinline__ void run_mix_ops(const DevOp* __restrict__ ops, const double* __restrict__ coef,
                                            const uint32_t* __restrict__ pool, uint32_t op0, uint32_t op1, bool rev,
                                            uint32_t jl, uint32_t jstep, bool active, uint32_t parb, Left left,
                                            Right right, const double2* __restrict__ icoef = nullptr,
                                            Sync sync = Sync()) {
  const uint32_t n = op1 - op0;
  if (n == 0) return;
  auto at = [&](uint32_t i) { return rev ? op1 - 1 - i : op0 + i; };
  auto first_of = [&](const DevOp& d) -> uint2 {
    return jl < d.count ? ldm<G>(reinterpret_cast<const uint2*>(pool + d.tab) + jl) : make_uint2(0u, 0u);
  };
  OpR<R> op = load_op<R, G>(ops, coef, at(0), icoef);
  uint2 first = first_of(op.d);
  for (uint32_t i = 0; i < n; ++i) {
    OpR<R> opn = op;
    uint2 firstn = make_uint2(0u, 0u);
    if (i + 1 < n) {
      opn = load_op<R, G>(ops, coef, at(i + 1), icoef);
      firstn = first_of(opn.d);
    }
    if (active) {
      const uint2* __restrict__ t = reinterpret_cast<const uint2*>(pool + op.d.tab);
      uint2 x = first;
      for (uint32_t j = jl; j < op.d.count; j += jstep) {
        const uint32_t jn = j + jstep;
        const uint2 xn = jn < op.d.count ? ldm<G>(t + jn) : make_uint2(0u, 0u);
        pair_update<A>(left(x.x & 0x7fffffffu), right(x.y), op.k, (x.x >> 31) ^ parb);
        x = xn;
      }
    }
    sync();
    op = opn;
    first = firstn;
  }
}

// The terms of a column-pair tile in chunks (one tile per CTA or per warp, one
// pair update per thread and trip): the descriptors, coefficients, table
// entries and element addresses of kPairChunk terms, kPairTrips trips each, are
// loaded and computed before the chunk's first update, so that a term costs its
// shared-memory loads, arithmetic, stores and barrier, not a chain of dependent
// global loads. Only inline pair matrices take this form (every term of the
// reference's getters); a chunk with another term, or with more entries than
// kPairTrips trips cover, runs through run_mix_ops. The update is pair_update's
// reduced form, bit for bit.

// G: descriptors and tables in global memory (read through the read-only
// cache); false when the caller has staged them in shared memory (a pass image).
template <typename R, class A, bool G = true, class Left, class Right, class Sync>
__device__ __forceinline__ void chunked_mix_ops(const DevOp* __restrict__ ops, const double* __restrict__ coef,
                                                const uint32_t* __restrict__ pool, uint32_t op0, uint32_t op1,
                                                bool rev, uint32_t jl, uint32_t jstep, bool active, uint32_t parb,
                                                Left left, Right right, const double2* __restrict__ icoef, Sync sync) {
  using C2 = typename Cx<R>::T;
  const uint32_t n = op1 - op0;
  // The terms of a MIX pass share one table length (pairs of alpha strings for
  // one excitation): passes whose tables need more trips skip the chunked form.
  if (n == 0) return;
  if (ldm<G>(reinterpret_cast<const uint4*>(ops + op0)).y > kPairTrips * jstep) {
    run_mix_ops<R, A, G>(ops, coef, pool, op0, op1, rev, jl, jstep, active, parb, left, right, icoef, sync);
    return;
  }
  for (uint32_t i0 = 0; i0 < n; i0 += kPairChunk) {
    const uint32_t m = min(kPairChunk, n - i0);
    R cc[kPairChunk], tt[kPairChunk];
    C2* lp[kPairChunk][kPairTrips];
    C2* rp[kPairChunk][kPairTrips];
    uint32_t par[kPairChunk];  // bit tr: parity of trip tr
    uint32_t okm[kPairChunk];  // bit tr: trip tr has an entry
    bool fast = true;
#pragma unroll
    for (uint32_t k = 0; k < kPairChunk; ++k) {
      cc[k] = tt[k] = (R)0;
      par[k] = okm[k] = 0;
#pragma unroll
      for (uint32_t tr = 0; tr < kPairTrips; ++tr) lp[k][tr] = rp[k][tr] = nullptr;
      if (k < m) {
        const uint32_t o = rev ? op1 - 1 - (i0 + k) : op0 + i0 + k;
        const uint4* src = reinterpret_cast<const uint4*>(ops + o);
        const uint4 a = ldm<G>(src), b = ldm<G>(src + 1);
        fast = fast && a.w == OP_INLINE && (a.z & 0xffu) == (uint32_t)OPK_PAIR && a.y <= kPairTrips * jstep;
        double c0 = __hiloint2double((int)b.y, (int)b.x), c1 = __hiloint2double((int)b.w, (int)b.z);
        if (icoef) {
          const double2 ic = __ldg(icoef + o);
          c0 = ic.x;
          c1 = ic.y;
        }
        cc[k] = (R)c0;
        tt[k] = (R)c1;
#pragma unroll
        for (uint32_t tr = 0; tr < kPairTrips; ++tr) {
          const uint32_t j = jl + tr * jstep;
          if (active && j < a.y) {
            const uint2 x = ldm<G>(reinterpret_cast<const uint2*>(pool + a.x) + j);
            lp[k][tr] = &left(x.x & 0x7fffffffu);
            rp[k][tr] = &right(x.y);
            par[k] |= (((x.x >> 31) ^ parb) & 1u) << tr;
            okm[k] |= 1u << tr;
          }
        }
      }
    }
    if (!fast) {
      run_mix_ops<R, A, G>(ops, coef, pool, rev ? op1 - (i0 + m) : op0 + i0, rev ? op1 - i0 : op0 + i0 + m, rev,
                              jl, jstep, active, parb, left, right, icoef, sync);
      continue;
    }
#pragma unroll
    for (uint32_t k = 0; k < kPairChunk; ++k) {
      if (k < m) {
#pragma unroll
        for (uint32_t tr = 0; tr < kPairTrips; ++tr) {
          if ((okm[k] >> tr) & 1u) {
            C2& l = *lp[k][tr];
            C2& r = *rp[k][tr];
            const C2 vl = l, vr = r;
            const R c = cc[k], t = ((par[k] >> tr) & 1u) ? neg(tt[k]) : tt[k];
            C2 nl, nr;
            nl.x = A::sub(A::mul(vl.x, c), A::mul(vr.y, t));
            nl.y = A::add(A::mul(vl.y, c), A::mul(vr.x, t));
            nr.x = A::sub(A::mul(vr.x, c), A::mul(vl.y, t));
            nr.y = A::add(A::mul(vl.x, t), A::mul(vr.y, c));
            l = nl;
            r = nr;
          }
        }
        sync();
      }
    }
  }
}

// The terms of a row or column tile (run_line_ops' layout: thread entries jl,
// jl + jstep, ... of each term on its own line) in chunks, like
// chunked_mix_ops: the descriptors of kPairChunk terms are loaded first, and
// when all of them are inline with at most kPairTrips trips, their table entries
// and element addresses follow before the first update. Pair terms take
// pair_update's reduced form, diagonal terms diag_update, bit for bit; a line
// whose string fails a term's conditions skips it. Any other chunk runs through
// run_line_ops.
template <typename R, class A, class Elem, class Sync>
__device__ __forceinline__ void chunked_line_ops(const DevOp* __restrict__ ops, const double* __restrict__ coef,
                                                 const uint32_t* __restrict__ pool, uint32_t op0, uint32_t op1,
                                                 bool rev, uint32_t L, uint32_t jl, uint32_t jstep, bool active,
                                                 uint32_t lstr, Elem elem, const double2* __restrict__ icoef,
                                                 Sync sync) {
  using C2 = typename Cx<R>::T;
  const uint32_t n = op1 - op0;
  for (uint32_t i0 = 0; i0 < n; i0 += kPairChunk) {
    const uint32_t m = min(kPairChunk, n - i0);
    uint4 da[kPairChunk];
    R cc[kPairChunk], tt[kPairChunk];
    bool fast = true;
#pragma unroll
    for (uint32_t k = 0; k < kPairChunk; ++k) {
      // Every slot's descriptor is loaded (at a clamped index), so that the
      // chunk's loads go out together instead of one after another behind guards.
      const uint32_t o = rev ? op1 - 1 - (i0 + min(k, m - 1)) : op0 + i0 + min(k, m - 1);
      const uint4* src = reinterpret_cast<const uint4*>(ops + o);
      const uint4 a = __ldg(src), b = __ldg(src + 1);
      const uint32_t kind = a.z & 0xffu;
      const uint32_t count = kind == OPK_DIAG_ALL ? L : a.y;
      if (k < m) fast = fast && a.w == OP_INLINE && count <= kPairTrips * jstep;
      double c0 = __hiloint2double((int)b.y, (int)b.x), c1 = __hiloint2double((int)b.w, (int)b.z);
      if (icoef) {
        const double2 ic = __ldg(icoef + o);
        c0 = ic.x;
        c1 = ic.y;
      }
      da[k] = a;
      cc[k] = (R)c0;
      tt[k] = (R)c1;
    }
    if (!fast) {
      run_line_ops<R, A, true>(ops, coef, pool, rev ? op1 - (i0 + m) : op0 + i0, rev ? op1 - i0 : op0 + i0 + m, rev,
                               L, jl, jstep, active, lstr, elem, icoef, sync);
      continue;
    }
    C2* p1[kPairChunk][kPairTrips];
    C2* p2[kPairChunk][kPairTrips];
    uint32_t par[kPairChunk];  // bit tr: parity of trip tr (pairs)
    uint32_t okm[kPairChunk];  // bit tr: trip tr has an entry on a line the term acts on
#pragma unroll
    for (uint32_t k = 0; k < kPairChunk; ++k) {
      par[k] = okm[k] = 0;
#pragma unroll
      for (uint32_t tr = 0; tr < kPairTrips; ++tr) p1[k][tr] = p2[k][tr] = nullptr;
      {
        const uint4 a = da[k];  // slots past the chunk hold its last term (loads only)
        const uint32_t kind = a.z & 0xffu, nc = (a.z >> 8) & 0xffu;
        uint32_t cm = 0;
        if (nc > 0) cm |= 1u << ((a.z >> 16) & 0xffu);
        if (nc > 1) cm |= 1u << (a.z >> 24);
        const bool on = k < m && active && (lstr & cm) == cm;
        const uint32_t count = kind == OPK_DIAG_ALL ? L : a.y;
#pragma unroll
        for (uint32_t tr = 0; tr < kPairTrips; ++tr) {
          const uint32_t j = jl + tr * jstep;
          // entries loaded at clamped indices as well; an empty table is not read
          const uint32_t jj = count ? min(j, count - 1) : 0u;
          const uint32_t* t = count ? pool + a.x : pool;
          if (kind == OPK_PAIR) {
            const uint2 x = __ldg(reinterpret_cast<const uint2*>(t) + jj);
            if (on && j < count) {
              p1[k][tr] = &elem(x.x & 0x7fffffffu);
              p2[k][tr] = &elem(x.y);
              par[k] |= (x.x >> 31) << tr;
              okm[k] |= 1u << tr;
            }
          } else {
            const uint32_t e = kind == OPK_DIAG_LIST ? __ldg(t + jj) : jj;
            if (on && j < count) {
              p1[k][tr] = &elem(e);
              okm[k] |= 1u << tr;
            }
          }
        }
      }
    }
#pragma unroll
    for (uint32_t k = 0; k < kPairChunk; ++k) {
      if (k < m) {
        const bool pair = (da[k].z & 0xffu) == OPK_PAIR;
#pragma unroll
        for (uint32_t tr = 0; tr < kPairTrips; ++tr) {
          if ((okm[k] >> tr) & 1u) {
            if (pair) {
              C2& l = *p1[k][tr];
              C2& r = *p2[k][tr];
              const C2 vl = l, vr = r;
              const R c = cc[k], t = ((par[k] >> tr) & 1u) ? neg(tt[k]) : tt[k];
              C2 nl, nr;
              nl.x = A::sub(A::mul(vl.x, c), A::mul(vr.y, t));
              nl.y = A::add(A::mul(vl.y, c), A::mul(vr.x, t));
              nr.x = A::sub(A::mul(vr.x, c), A::mul(vl.y, t));
              nr.y = A::add(A::mul(vl.x, t), A::mul(vr.y, c));
              l = nl;
              r = nr;
            } else {
              C2& v = *p1[k][tr];
              R xr, xi;
              cmul<A>(v.x, v.y, cc[k], tt[k], xr, xi);
              v.x = xr;
              v.y = xi;
            }
          }
        }
        sync();
      }
    }
  }
}

}  // namespace qpe

#endif  // QPE_TILE_OPS_CUH_
