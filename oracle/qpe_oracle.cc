// qpe_oracle.cc - CPU restatement of qpe-sim's hot path.
//
// TEST INFRASTRUCTURE ONLY. This file is the oracle: tests/, __graft_entry__.smoke()
// and bench.py's CPU-baseline leg call it as the checker. The product path never
// links or calls it.
//
// It restates, in plain C++ with OpenMP, the reference's algorithm for the
// controlled Trotterized evolution, the QIFT and the phase histogram; each
// function names the reference file:line it follows. Parity pins: the reference
// itself, compiled from its own sources with project-written shims (oracle/_ref,
// see oracle/Makefile), produced the golden vectors under tests/golden/ that the
// CPU test suite checks this file against.
//
// Extension beyond the reference (labelled): n_alpha != n_beta (odd electron
// counts). The reference has one occupation count for both spins
// (cpp/time_evolution_over_terms.hpp:159-167); with n_alpha == n_beta this file
// reproduces it, otherwise it applies the same tables per spin with that spin's
// count. That case is "parity unpinned" by the reference.
#include <algorithm>
#include <cmath>
#include <complex>
#include <cstdint>
#include <cstring>
#include <vector>

#ifdef _OPENMP
#include <omp.h>
#endif

#include "../include/qpe_gb300.h"
#include "dft_fp64.h"

namespace orc {

using cplx = std::complex<double>;

// cpp/util.hpp:49-60 (including its behaviour for negative k, which the
// incremental-rank tables of cpp/offset_computer.hpp:85-86 rely on).
static inline uint64_t nck(int n, int k) {
  if (k > n) return 0;
  if (k * 2 > n) k = n - k;
  if (k == 0) return 1;
  uint64_t r = (uint64_t)n;
  for (int i = 2; i <= k; ++i) {
    r *= (uint64_t)(n - i + 1);
    r /= (uint64_t)i;
  }
  return r;
}

// cpp/offset_computer.hpp:16-27: colex rank, sum over set bits of C(pos, order).
static inline int64_t rank(uint64_t bv) {
  int64_t acc = 0;
  unsigned order = 1;
  for (unsigned pos = 0; bv != 0; ++pos, bv >>= 1) {
    if (bv & 1) {
      acc += (int64_t)nck((int)pos, (int)order);
      ++order;
    }
  }
  return acc;
}

// cpp/util.hpp:62-70: next bit string of the same weight in colex order.
static inline uint64_t next_comb(uint64_t x) {
  uint64_t lowest = x & (0 - x);
  uint64_t ripple = x + lowest;
  return ripple + (((ripple ^ x) / lowest) >> 2);
}

// cpp/util.hpp:73-81: parity by xor folding.
static inline unsigned parity(uint64_t x) {
  x ^= x >> 32;
  x ^= x >> 16;
  x ^= x >> 8;
  x ^= x >> 4;
  x ^= x >> 2;
  x ^= x >> 1;
  return (unsigned)(x & 1);
}

static inline unsigned popcount(uint64_t x) {
  unsigned c = 0;
  for (; x; x &= x - 1) ++c;
  return c;
}

// ---------------------------------------------------------------------------
// Run tables: cpp/time_evolution_over_terms.hpp:19-25 (MixedPQRSLoopInfo) and the
// discover*_BVs routines (:1160-1411). A run is a set of free-bit strings that
// differ only below the lowest fixed orbital; their ranks are contiguous, so a run
// is stored as (off01, off10, niter, mid_parity).
struct Run {
  uint64_t niter;
  uint64_t off01;
  uint64_t off10;
  unsigned mid_parity;
};

// Inserts a zero bit at each (ascending) fixed position, i.e. spreads the free
// bits around the term's orbitals (the lo/mid/hi segments of :1176-1184).
static inline uint64_t spread(uint64_t free_bits, const unsigned* fixed, int nfixed) {
  uint64_t out = free_bits;
  for (int i = 0; i < nfixed; ++i) {
    uint64_t low = out & ((1ull << fixed[i]) - 1);
    out = low | ((out >> fixed[i]) << (fixed[i] + 1));
  }
  return out;
}

// Bits of `full` strictly between positions lo and hi.
static inline uint64_t between(uint64_t full, unsigned lo, unsigned hi) {
  if (hi <= lo + 1) return 0;
  return (full >> (lo + 1)) & ((1ull << (hi - lo - 1)) - 1);
}

enum AxisKind { AX_N = 0, AX_NN, AX_CA, AX_CNA, AX_CCAA };

// One routine for the five discover functions. `count` is the table length the
// reference sizes its vector with (e.g. e2_of_n4 for CCAA, :846); the loop walks
// next_comb from the smallest string of weight `w`, emitting one run per distinct
// configuration of the bits above the lowest fixed orbital.
//   N    (q)          :1374-1411   occupied: q
//   NN   (p, r)       :1335-1372   occupied: p, r
//   CA   (p, r)       :1279-1333   01 side r occupied, 10 side p occupied
//   CNA  (p, q, r)    :1217-1277   q occupied; 01 side r, 10 side p
//   CCAA (p, q, r, s) :1160-1215   01 side r, s; 10 side p, q
static std::vector<Run> discover(AxisKind kind, unsigned M, unsigned e, unsigned p, unsigned q,
                                 unsigned r, unsigned s) {
  unsigned fixed[4];
  int nf = 0;
  int n_occ_fixed = 0;
  switch (kind) {
    case AX_N: fixed[0] = q; nf = 1; n_occ_fixed = 1; break;
    case AX_NN: fixed[0] = p; fixed[1] = r; nf = 2; n_occ_fixed = 2; break;
    case AX_CA: fixed[0] = p; fixed[1] = r; nf = 2; n_occ_fixed = 1; break;
    case AX_CNA: fixed[0] = p; fixed[1] = q; fixed[2] = r; nf = 3; n_occ_fixed = 2; break;
    case AX_CCAA: fixed[0] = p; fixed[1] = q; fixed[2] = r; fixed[3] = s; nf = 4; n_occ_fixed = 2; break;
  }
  std::sort(fixed, fixed + nf);
  const int w = (int)e - n_occ_fixed;
  // The reference computes these counts from unsigned globals converted to int,
  // so a negative size argument yields 0 through nChoosek's k > n test.
  const uint64_t count = nck((int)M - nf, w);
  std::vector<Run> runs;
  if (count == 0 || w < 0) return runs;
  uint64_t ctr = 0;
  uint64_t bv = (w == 0) ? 0 : ((1ull << w) - 1);
  while (ctr < count) {
    const uint64_t base = spread(bv, fixed, nf);
    Run run{};
    switch (kind) {
      case AX_N: run.off01 = run.off10 = (uint64_t)rank(base | (1ull << q)); break;
      case AX_NN: run.off01 = (uint64_t)rank(base | (1ull << p) | (1ull << r)); break;  // off10 unset (:1353)
      case AX_CA: {
        run.off01 = (uint64_t)rank(base | (1ull << r));
        run.off10 = (uint64_t)rank(base | (1ull << p));
        run.mid_parity = parity(between(base, std::min(p, r), std::max(p, r)));
        break;
      }
      case AX_CNA: {
        run.off01 = (uint64_t)rank(base | (1ull << q) | (1ull << r));
        run.off10 = (uint64_t)rank(base | (1ull << q) | (1ull << p));
        // :1240-1251: parity of the occupied orbitals strictly between p and r,
        // counting q when it lies between them.
        if (q > r)
          run.mid_parity = parity(between(base, p, r));
        else if (q < p)
          run.mid_parity = parity(between(base, p, r));
        else
          run.mid_parity = parity(between(base, p, q)) + parity(between(base, q, r)) + 1;
        break;
      }
      case AX_CCAA: {
        run.off01 = (uint64_t)rank(base | (1ull << r) | (1ull << s));
        run.off10 = (uint64_t)rank(base | (1ull << q) | (1ull << p));
        // :1187: parity(midlo) + parity(midhi) over the sorted orbitals.
        run.mid_parity = parity(between(base, fixed[0], fixed[1])) +
                         parity(between(base, fixed[2], fixed[3]));
        break;
      }
    }
    const uint64_t lo = bv & ((1ull << fixed[0]) - 1);
    uint64_t niter = 1;
    if (lo != 0) niter = nck((int)fixed[0], (int)popcount(lo));
    run.niter = niter;
    runs.push_back(run);
    ctr += niter;
    bv = (bv == 0) ? 1 : bv;
    for (uint64_t i = 0; i < niter; ++i) bv = next_comb(bv);
  }
  return runs;
}

// ---------------------------------------------------------------------------
// State geometry and the pair-update primitives.
struct Geom {
  unsigned M, ea, eb;
  uint64_t Ca, Cb, block;
};

// Touch counting (orc_touches_per_power): while set, every update primitive adds
// the amplitude updates it would make (2 per pair, 1 per diagonal phase) and
// returns without touching the block.
static uint64_t* g_touches = nullptr;

static uint64_t run_total(const std::vector<Run>& r) {
  uint64_t n = 0;
  for (const Run& x : r) n += x.niter;
  return n;
}

static inline void coeffs_of(const qpe_term& t, unsigned par, cplx& c0, cplx& c1) {
  const double* m = (par & 1) ? t.odd : t.even;
  c0 = cplx(m[0], m[1]);
  c1 = cplx(m[2], m[3]);
}

// cpp/time_evolution_over_terms.hpp:565-589.
static inline void pair_update(cplx* sv, const cplx& c0, const cplx& c1, uint64_t l, uint64_t r) {
  const cplx vl = sv[l];
  const cplx vr = sv[r];
  sv[l] = vl * c0 + vr * c1;
  sv[r] = vl * c1 + vr * c0;
}

// Row-pair x all-columns update (_updateAAAA :591-659 and updatePQ_AA :927-958).
static void rows_pairs_all_cols(cplx* blk, const Geom& g, const std::vector<Run>& ra,
                                const qpe_term& t) {
  if (g_touches) {
    *g_touches += 2 * run_total(ra) * g.Cb;
    return;
  }
  std::vector<uint64_t> goal(ra.size() + 1, 0);
  for (size_t i = 0; i < ra.size(); ++i) goal[i + 1] = goal[i] + ra[i].niter;
  const int64_t total = (int64_t)goal.back();
#pragma omp parallel for schedule(guided)
  for (int64_t pos = 0; pos < total; ++pos) {
    const size_t run = (size_t)(std::upper_bound(goal.begin(), goal.end(), (uint64_t)pos) - goal.begin()) - 1;
    const uint64_t off = (uint64_t)pos - goal[run];
    cplx c0, c1;
    coeffs_of(t, ra[run].mid_parity, c0, c1);
    const uint64_t l0 = (ra[run].off01 + off) * g.Cb;
    const uint64_t r0 = (ra[run].off10 + off) * g.Cb;
    for (uint64_t b = 0; b < g.Cb; ++b) pair_update(blk, c0, c1, l0 + b, r0 + b);
  }
}

// All-rows x column-pair update (_updateBBBB :661-735 and updatePQ_BB :959-986).
static void all_rows_cols_pairs(cplx* blk, const Geom& g, const std::vector<Run>& rb,
                                const qpe_term& t) {
  if (g_touches) {
    *g_touches += 2 * g.Ca * run_total(rb);
    return;
  }
#pragma omp parallel for schedule(static)
  for (int64_t a = 0; a < (int64_t)g.Ca; ++a) {
    const uint64_t row = (uint64_t)a * g.Cb;
    for (const Run& run : rb) {
      cplx c0, c1;
      coeffs_of(t, run.mid_parity, c0, c1);
      for (uint64_t i = 0; i < run.niter; ++i)
        pair_update(blk, c0, c1, row + run.off01 + i, row + run.off10 + i);
    }
  }
}

// Row-pair x column-pair (or column-list) update (_updateABBA :737-839): the
// parity is the sum of both sides' run parities (:774).
static void rows_pairs_cols_runs(cplx* blk, const Geom& g, const std::vector<Run>& ra,
                                 const std::vector<Run>& rb, const qpe_term& t) {
  if (g_touches) {
    *g_touches += 2 * run_total(ra) * run_total(rb);
    return;
  }
  std::vector<uint64_t> goal(ra.size() + 1, 0);
  for (size_t i = 0; i < ra.size(); ++i) goal[i + 1] = goal[i] + ra[i].niter;
  const int64_t total = (int64_t)goal.back();
#pragma omp parallel for
  for (int64_t pos = 0; pos < total; ++pos) {
    const size_t run = (size_t)(std::upper_bound(goal.begin(), goal.end(), (uint64_t)pos) - goal.begin()) - 1;
    const uint64_t off = (uint64_t)pos - goal[run];
    const uint64_t l0 = (ra[run].off01 + off) * g.Cb;
    const uint64_t r0 = (ra[run].off10 + off) * g.Cb;
    for (const Run& bb : rb) {
      cplx c0, c1;
      coeffs_of(t, 1 & (ra[run].mid_parity + bb.mid_parity), c0, c1);
      for (uint64_t i = 0; i < bb.niter; ++i) pair_update(blk, c0, c1, l0 + bb.off01 + i, r0 + bb.off10 + i);
    }
  }
}

// Row-list x column-pair update (updatePQQR_BAAB :1109-1158).
static void rows_list_cols_pairs(cplx* blk, const Geom& g, const std::vector<Run>& ra,
                                 const std::vector<Run>& rb, const qpe_term& t) {
  if (g_touches) {
    *g_touches += 2 * run_total(ra) * run_total(rb);
    return;
  }
#pragma omp parallel for
  for (int64_t ia = 0; ia < (int64_t)ra.size(); ++ia) {
    for (uint64_t na = 0; na < ra[ia].niter; ++na) {
      const uint64_t row = (ra[ia].off01 + na) * g.Cb;
      for (const Run& bb : rb) {
        cplx c0, c1;
        coeffs_of(t, bb.mid_parity, c0, c1);
        for (uint64_t i = 0; i < bb.niter; ++i) pair_update(blk, c0, c1, row + bb.off01 + i, row + bb.off10 + i);
      }
    }
  }
}

// Diagonal phase on row-list x all columns (updatePP_AA :886-906, updatePQQP_AA :988-1014).
static void diag_rows(cplx* blk, const Geom& g, const std::vector<Run>& ra, const cplx& c) {
  if (g_touches) {
    *g_touches += run_total(ra) * g.Cb;
    return;
  }
#pragma omp parallel for
  for (int64_t ia = 0; ia < (int64_t)ra.size(); ++ia)
    for (uint64_t na = 0; na < ra[ia].niter; ++na) {
      const uint64_t row = (ra[ia].off01 + na) * g.Cb;
      for (uint64_t b = 0; b < g.Cb; ++b) blk[row + b] *= c;
    }
}

// Diagonal phase on all rows x column-list (updatePP_BB :907-925, updatePQQP_BB :1015-1039).
static void diag_cols(cplx* blk, const Geom& g, const std::vector<Run>& rb, const cplx& c) {
  if (g_touches) {
    *g_touches += g.Ca * run_total(rb);
    return;
  }
#pragma omp parallel for
  for (int64_t a = 0; a < (int64_t)g.Ca; ++a) {
    const uint64_t row = (uint64_t)a * g.Cb;
    for (const Run& bb : rb)
      for (uint64_t i = 0; i < bb.niter; ++i) blk[row + bb.off01 + i] *= c;
  }
}

// Diagonal phase on row-list x column-list (updatePQQP_AB :1040-1071).
static void diag_rows_cols(cplx* blk, const Geom& g, const std::vector<Run>& ra,
                           const std::vector<Run>& rb, const cplx& c) {
  if (g_touches) {
    *g_touches += run_total(ra) * run_total(rb);
    return;
  }
#pragma omp parallel for
  for (int64_t ia = 0; ia < (int64_t)ra.size(); ++ia)
    for (uint64_t na = 0; na < ra[ia].niter; ++na) {
      const uint64_t row = (ra[ia].off01 + na) * g.Cb;
      for (const Run& bb : rb)
        for (uint64_t i = 0; i < bb.niter; ++i) blk[row + bb.off01 + i] *= c;
    }
}

// ---------------------------------------------------------------------------
// Per-term dispatch on spin class (the branches inside applyUnitary_reordered).
static void apply_pp(cplx* blk, const Geom& g, const qpe_term& t) {
  const cplx c(t.even[0], t.even[1]);
  if (t.p < g.M)
    diag_rows(blk, g, discover(AX_N, g.M, g.ea, 0, t.p, 0, 0), c);          // :386-390
  else
    diag_cols(blk, g, discover(AX_N, g.M, g.eb, 0, t.p - g.M, 0, 0), c);    // :391-395
}

static void apply_pqqp(cplx* blk, const Geom& g, const qpe_term& t) {
  const cplx c(t.even[0], t.even[1]);
  const unsigned p = t.p, q = t.q;
  if (p < g.M && q < g.M) {  // :411-414, updatePQQP_AA returns for e < 2 (:991-994)
    if (g.ea < 2) return;
    diag_rows(blk, g, discover(AX_NN, g.M, g.ea, p, 0, q, 0), c);
  } else if (p >= g.M && q >= g.M) {
    if (g.eb < 2) return;
    diag_cols(blk, g, discover(AX_NN, g.M, g.eb, p - g.M, 0, q - g.M, 0), c);
  } else {
    diag_rows_cols(blk, g, discover(AX_N, g.M, g.ea, 0, p, 0, 0), discover(AX_N, g.M, g.eb, 0, q - g.M, 0, 0), c);
  }
}

static void apply_pq(cplx* blk, const Geom& g, const qpe_term& t) {
  const unsigned p = t.p, q = t.q;
  if (p < g.M && q < g.M)  // :441-445 -> updatePQ_AA: discoverCA(p, q)
    rows_pairs_all_cols(blk, g, discover(AX_CA, g.M, g.ea, p, 0, q, 0), t);
  else  // :446-450 -> updatePQ_BB
    all_rows_cols_pairs(blk, g, discover(AX_CA, g.M, g.eb, p - g.M, 0, q - g.M, 0), t);
}

static void apply_pqqr(cplx* blk, const Geom& g, const qpe_term& t) {
  // key (p, q, q, r): t.p = p, t.q = q, t.s = r (the reference unpacks p, q, garb, r).
  const unsigned p = t.p, q = t.q, r = t.s;
  if (p < g.M && q < g.M) {  // AAAA :1073-1085
    if (g.ea < 2) return;
    rows_pairs_all_cols(blk, g, discover(AX_CNA, g.M, g.ea, p, q, r, 0), t);
  } else if (p >= g.M && q >= g.M) {  // BBBB :1086-1098
    if (g.eb < 2) return;
    all_rows_cols_pairs(blk, g, discover(AX_CNA, g.M, g.eb, p - g.M, q - g.M, r - g.M, 0), t);
  } else if (q >= g.M) {  // ABBA :1099-1107: alpha CA(p, r), beta N(q)
    rows_pairs_cols_runs(blk, g, discover(AX_CA, g.M, g.ea, p, 0, r, 0),
                         discover(AX_N, g.M, g.eb, 0, q - g.M, 0, 0), t);
  } else {  // BAAB :1109-1158: alpha N(q), beta CA(p, r)
    rows_list_cols_pairs(blk, g, discover(AX_N, g.M, g.ea, 0, q, 0, 0),
                         discover(AX_CA, g.M, g.eb, p - g.M, 0, r - g.M, 0), t);
  }
}

static void apply_pqrs(cplx* blk, const Geom& g, const qpe_term& t) {
  const unsigned p = t.p, q = t.q, r = t.r, s = t.s;
  if (p < g.M && q < g.M && r < g.M && s < g.M) {  // AAAA :841-857
    if (g.ea < 2) return;
    rows_pairs_all_cols(blk, g, discover(AX_CCAA, g.M, g.ea, p, q, r, s), t);
  } else if (p >= g.M && q >= g.M && r >= g.M && s >= g.M) {  // BBBB :859-870
    if (g.eb < 2) return;
    all_rows_cols_pairs(blk, g, discover(AX_CCAA, g.M, g.eb, p - g.M, q - g.M, r - g.M, s - g.M), t);
  } else {  // ABBA :872-884: alpha CA(p, s), beta CA(q, r)
    rows_pairs_cols_runs(blk, g, discover(AX_CA, g.M, g.ea, p, 0, s, 0),
                         discover(AX_CA, g.M, g.eb, q - g.M, 0, r - g.M, 0), t);
  }
}

struct Terms {
  const qpe_term *pp, *pq, *pqqp, *pqqr, *pqrs;
  size_t npp, npq, npqqp, npqqr, npqrs;
};

// applyUnitary_reordered (:374-562): pp, pqqp, then each pq followed by every pqqr
// (p_, q_, q_, r_) with p_ == q and r_ == p (:465), then pqrs.
static void sweep(cplx* blk, const Geom& g, const Terms& T, bool reversed) {
  // The reversed sweep (second-order extension) replays the same term list
  // backwards; the first-order sweep is the reference's.
  struct Item { int kind; const qpe_term* t; };
  std::vector<Item> seq;
  for (size_t i = 0; i < T.npp; ++i) seq.push_back({QPE_TERM_PP, &T.pp[i]});
  for (size_t i = 0; i < T.npqqp; ++i) seq.push_back({QPE_TERM_PQQP, &T.pqqp[i]});
  for (size_t i = 0; i < T.npq; ++i) {
    seq.push_back({QPE_TERM_PQ, &T.pq[i]});
    for (size_t j = 0; j < T.npqqr; ++j)
      if (T.pqqr[j].p == T.pq[i].q && T.pqqr[j].s == T.pq[i].p) seq.push_back({QPE_TERM_PQQR, &T.pqqr[j]});
  }
  for (size_t i = 0; i < T.npqrs; ++i) seq.push_back({QPE_TERM_PQRS, &T.pqrs[i]});
  if (reversed) std::reverse(seq.begin(), seq.end());
  for (const Item& it : seq) {
    switch (it.kind) {
      case QPE_TERM_PP: apply_pp(blk, g, *it.t); break;
      case QPE_TERM_PQQP: apply_pqqp(blk, g, *it.t); break;
      case QPE_TERM_PQ: apply_pq(blk, g, *it.t); break;
      case QPE_TERM_PQQR: apply_pqqr(blk, g, *it.t); break;
      case QPE_TERM_PQRS: apply_pqrs(blk, g, *it.t); break;
    }
  }
}

// applyUnitary (:174-372), the order of the iterative variant: every pp, every
// pq, every pqqp, every pqqr (no nesting and no skipping), every pqrs.
static void sweep_apply_unitary(cplx* blk, const Geom& g, const Terms& T) {
  for (size_t i = 0; i < T.npp; ++i) apply_pp(blk, g, T.pp[i]);
  for (size_t i = 0; i < T.npq; ++i) apply_pq(blk, g, T.pq[i]);
  for (size_t i = 0; i < T.npqqp; ++i) apply_pqqp(blk, g, T.pqqp[i]);
  for (size_t i = 0; i < T.npqqr; ++i) apply_pqqr(blk, g, T.pqqr[i]);
  for (size_t i = 0; i < T.npqrs; ++i) apply_pqrs(blk, g, T.pqrs[i]);
}

}  // namespace orc

using namespace orc;

extern "C" {

int orc_version(void) { return 1; }

uint64_t orc_nchoosek(int n, int k) { return nck(n, k); }
int64_t orc_rank(uint64_t bv) { return rank(bv); }
uint64_t orc_next_comb(uint64_t x) { return next_comb(x); }
unsigned orc_parity(uint64_t x) { return parity(x); }

// Writes the run table of one discover routine; returns the run count, or -1 if
// cap is too small. kind: 0 N, 1 NN, 2 CA, 3 CNA, 4 CCAA.
int64_t orc_discover(int kind, unsigned M, unsigned e, unsigned p, unsigned q, unsigned r, unsigned s,
                     uint64_t* niter, uint64_t* off01, uint64_t* off10, unsigned* mid_parity, size_t cap) {
  std::vector<Run> runs = discover((AxisKind)kind, M, e, p, q, r, s);
  if (runs.size() > cap) return -1;
  for (size_t i = 0; i < runs.size(); ++i) {
    niter[i] = runs[i].niter;
    off01[i] = runs[i].off01;
    off10[i] = runs[i].off10;
    mid_parity[i] = runs[i].mid_parity;
  }
  return (int64_t)runs.size();
}

// time_evolve_over_terms (:92-139) over blocks [first, last): copy block k-1 to
// block k (:130-132), then one power of U. order 2 applies a forward and a
// reversed sweep; steps repeats the step (both extensions; 1, 1 = reference).
int orc_time_evolve(unsigned M, unsigned ea, unsigned eb, unsigned P, const qpe_term* pp, size_t npp,
                    const qpe_term* pq, size_t npq, const qpe_term* pqqp, size_t npqqp, const qpe_term* pqqr,
                    size_t npqqr, const qpe_term* pqrs, size_t npqrs, unsigned order, unsigned steps,
                    unsigned first, unsigned last, double* state) {
  if (M == 0 || M > 31 || ea > M || eb > M || P == 0 || P > 30) return QPE_ERR_INVALID;
  Geom g{M, ea, eb, nck((int)M, (int)ea), nck((int)M, (int)eb), 0};
  g.block = g.Ca * g.Cb;
  const uint64_t nblocks = 1ull << P;
  if (first == 0 && last == 0) { first = 1; last = (unsigned)nblocks; }
  if (first < 1 || last > nblocks || first > last) return QPE_ERR_INVALID;
  Terms T{pp, pq, pqqp, pqqr, pqrs, npp, npq, npqqp, npqqr, npqrs};
  cplx* sv = reinterpret_cast<cplx*>(state);
  for (uint64_t k = first; k < last; ++k) {
    cplx* blk = sv + k * g.block;
    std::memcpy(blk, sv + (k - 1) * g.block, sizeof(cplx) * g.block);
    for (unsigned st = 0; st < (steps ? steps : 1); ++st) {
      sweep(blk, g, T, false);
      if (order == 2) sweep(blk, g, T, true);
    }
  }
  return QPE_OK;
}

// Amplitude updates of one controlled power (order 2: a forward and a reversed
// sweep per step; `steps` steps): each primitive counts 2 per pair update and 1
// per diagonal phase, from the same run tables it would apply.
uint64_t orc_touches_per_power(unsigned M, unsigned ea, unsigned eb, const qpe_term* pp, size_t npp,
                               const qpe_term* pq, size_t npq, const qpe_term* pqqp, size_t npqqp,
                               const qpe_term* pqqr, size_t npqqr, const qpe_term* pqrs, size_t npqrs,
                               unsigned order, unsigned steps) {
  if (M == 0 || M > 31 || ea > M || eb > M) return 0;
  Geom g{M, ea, eb, nck((int)M, (int)ea), nck((int)M, (int)eb), 0};
  g.block = g.Ca * g.Cb;
  Terms T{pp, pq, pqqp, pqqr, pqrs, npp, npq, npqqp, npqqr, npqrs};
  uint64_t n = 0;
  g_touches = &n;
  sweep(nullptr, g, T, false);
  g_touches = nullptr;
  return n * (order == 2 ? 2 : 1) * (steps ? steps : 1);
}

// time_evolve_iqpe (:141-155): block 1 of the register, in place, receives
// `applications` sweeps of applyUnitary(..., exp = 1); no block is copied.
int orc_time_evolve_iqpe(unsigned M, unsigned ea, unsigned eb, unsigned P, const qpe_term* pp, size_t npp,
                         const qpe_term* pq, size_t npq, const qpe_term* pqqp, size_t npqqp, const qpe_term* pqqr,
                         size_t npqqr, const qpe_term* pqrs, size_t npqrs, unsigned applications, double* state) {
  if (M == 0 || M > 31 || ea > M || eb > M || P == 0 || P > 30) return QPE_ERR_INVALID;
  Geom g{M, ea, eb, nck((int)M, (int)ea), nck((int)M, (int)eb), 0};
  g.block = g.Ca * g.Cb;
  Terms T{pp, pq, pqqp, pqqr, pqrs, npp, npq, npqqp, npqqr, npqrs};
  cplx* blk = reinterpret_cast<cplx*>(state) + g.block;
  for (unsigned i = 0; i < applications; ++i) sweep_apply_unitary(blk, g, T);
  return QPE_OK;
}

// StateVector::qift (cpp/state_vector.hpp:115-179): forward DFT along the ancilla
// axis (stride ld, ld transforms, distance 1), then division by sqrt(N) (:172-178).
int orc_qift(unsigned P, uint64_t ld, double* state) {
  if (P == 0 || P > 30 || ld == 0) return QPE_ERR_INVALID;
  const uint64_t N = 1ull << P;
  dft_fp64::forward_strided(reinterpret_cast<std::complex<double>*>(state), N, ld, ld);
  const double norm = std::sqrt((double)N);
  cplx* sv = reinterpret_cast<cplx*>(state);
#pragma omp parallel for
  for (int64_t i = 0; i < (int64_t)(ld * N); ++i) sv[i] /= norm;
  return QPE_OK;
}

// StateVector::IdentifyPhaseAmplitudes (cpp/state_vector.hpp:341-372).
int orc_identify_phase_amplitudes(unsigned P, uint64_t ld, const double* state, double* probs) {
  if (P == 0 || P > 30 || ld == 0) return QPE_ERR_INVALID;
  const uint64_t N = 1ull << P;
  const cplx* sv = reinterpret_cast<const cplx*>(state);
#pragma omp parallel for
  for (int64_t k = 0; k < (int64_t)N; ++k) {
    double acc = 0;
    for (uint64_t off = 0; off < ld; ++off) acc += std::pow(std::abs(sv[(uint64_t)k * ld + off]), 2);
    probs[k] = acc;
  }
  return QPE_OK;
}

// ---------------------------------------------------------------------------
// OffsetComputer's incremental ranks (cpp/offset_computer.hpp:71-192), restated
// with the same prefix tables GEP/GEM (>= position) and GTP/GTM (> position).
struct Incr {
  unsigned n;
  int64_t bv_rank;
  std::vector<unsigned> bits, order;
  std::vector<int64_t> GEP[2], GEM[2], GTP[2], GTM[2];
  Incr(unsigned n_, uint64_t bv) : n(n_), bv_rank(rank(bv)), bits(n_, 0), order(n_, 0) {
    unsigned acc = 0;
    for (unsigned i = 0; i < n; ++i) {
      bits[i] = (bv >> i) & 1;
      acc += bits[i];
      order[i] = acc;
    }
    for (int v = 0; v < 2; ++v) {
      GEP[v].assign(n, 0); GEM[v].assign(n, 0); GTP[v].assign(n, 0); GTM[v].assign(n, 0);
      for (unsigned i = 0; i < n; ++i)
        if (bits[i]) {
          GEP[v][i] = -(int64_t)nck((int)i, (int)order[i]) + (int64_t)nck((int)i, (int)order[i] + (v + 1));
          GEM[v][i] = -(int64_t)nck((int)i, (int)order[i]) + (int64_t)nck((int)i, (int)order[i] - (v + 1));
        }
      for (int i = (int)n - 2; i >= 0; --i) {
        GEP[v][i] += GEP[v][i + 1];
        GEM[v][i] += GEM[v][i + 1];
      }
      for (int i = (int)n - 2; i >= 0; --i) {
        GTP[v][i] = GEP[v][i + 1];
        GTM[v][i] = GEM[v][i + 1];
      }
    }
  }
  int64_t plus(int N, unsigned lo, unsigned hi) const { return GTP[N - 1][lo] - GEP[N - 1][hi]; }
  int64_t minus(int N, unsigned lo, unsigned hi) const { return GTM[N - 1][lo] - GEM[N - 1][hi]; }
  int64_t destroy(unsigned b) const { return -(int64_t)nck((int)b, (int)order[b]); }
  int64_t create(unsigned b, int ord) const { return (int64_t)nck((int)b, ord); }
  int64_t swap1(unsigned i, unsigned j) const {
    if (bits[i] == bits[j]) return bv_rank;
    unsigned lo = std::min(i, j), hi = std::max(i, j);
    if (bits[lo] == 1) return bv_rank + destroy(lo) + create(hi, (int)order[hi]) + minus(1, lo, hi);
    return bv_rank + destroy(hi) + create(lo, (int)order[lo] + 1) + plus(1, lo, hi);
  }
  int64_t swap2(unsigned i, unsigned j, unsigned k, unsigned l) const {
    unsigned sum = bits[i] + bits[j] + bits[k] + bits[l];
    if (sum == 0 || sum == 4) return bv_rank;
    unsigned pos[4] = {i, j, k, l};
    std::sort(pos, pos + 4);
    unsigned config = bits[pos[0]] + (bits[pos[1]] << 1) + (bits[pos[2]] << 2) + (bits[pos[3]] << 3);
    int64_t v;
    switch (config) {
      case 0x3:
        v = bv_rank + minus(1, pos[0], pos[1]) + minus(2, pos[1], pos[2]) + minus(1, pos[2], pos[3]) +
            destroy(pos[0]) + destroy(pos[1]) + create(pos[2], (int)order[pos[2]] - 1) +
            create(pos[3], (int)order[pos[3]]);
        break;
      case 0x5: case 0x6: case 0x9: case 0xA:
        v = swap1(i, j) + swap1(k, l) - bv_rank;
        break;
      case 0xC:
        v = bv_rank + plus(1, pos[0], pos[1]) + plus(2, pos[1], pos[2]) + plus(1, pos[2], pos[3]) +
            destroy(pos[2]) + destroy(pos[3]) + create(pos[0], (int)order[pos[0]] + 1) +
            create(pos[1], (int)order[pos[1]] + 2);
        break;
      default:
        return -1;
    }
    // The reference stores this in an `unsigned` (:160) before returning it.
    return (int64_t)(uint32_t)v;
  }
};

// swaps: rows of 4 positions; a row whose last two entries are 0xFFFFFFFF is a
// single swap (rank_with_swap), otherwise a double swap.
int orc_rank_with_swaps(unsigned n, uint64_t bv, const uint32_t* swaps, int64_t* out, size_t nq) {
  if (n == 0 || n > 63) return QPE_ERR_INVALID;
  Incr oc(n, bv);
  for (size_t i = 0; i < nq; ++i) {
    const uint32_t* s = swaps + 4 * i;
    if (s[0] >= n || s[1] >= n) return QPE_ERR_INVALID;
    if (s[2] == 0xFFFFFFFFu)
      out[i] = oc.swap1(s[0], s[1]);
    else {
      if (s[2] >= n || s[3] >= n) return QPE_ERR_INVALID;
      out[i] = oc.swap2(s[0], s[1], s[2], s[3]);
    }
  }
  return QPE_OK;
}

void orc_set_threads(int n) {
#ifdef _OPENMP
  if (n > 0) omp_set_num_threads(n);
#else
  (void)n;
#endif
}

int orc_num_threads(void) {
#ifdef _OPENMP
  int n = 1;
#pragma omp parallel
  {
#pragma omp single
    n = omp_get_num_threads();
  }
  return n;
#else
  return 1;
#endif
}

}  // extern "C"
