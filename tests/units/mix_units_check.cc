// mix_units_check.cc - CPU check of the column-pair update-unit scheduler
// (2022-qpesim_gb300/csrc/mix_units.cpp), compiled with it by
// tests/test_mix_units.py.
//
// For a program built from the given terms it fills the pair tables the
// column-pair passes use (alpha and beta CA tables: every string with r occupied
// and p empty, paired with the string that moves the electron to p, with the
// parity of the occupied orbitals between them; ranks in colex order), builds the
// unit schedule and then, on a random complex128 block:
//   - applies every scheduled window the way the tile runner does (each pass,
//     each column pair, each term, each table entry in order),
//   - applies the same window the way k_resident_lean runs the warp programs
//     (gather into per-group stages, level by level, scatter back),
// and counts every difference between the two blocks (bit for bit) and every
// broken invariant the kernel relies on: a team of two or three warps is warps
// 0 .. tw - 1 of one group with equal headers; at most 64 amplitudes per warp;
// stage indices inside the group's stage and used by one team; rows and columns
// inside the block; each amplitude gathered at most once per window; every
// update inside its own team's amplitudes; the window's first term in w[1].
#include <cstdio>
#include <cstring>
#include <random>
#include <set>
#include <vector>

#include "mix_units.h"

using namespace qpe;

namespace {

uint32_t colex_rank(uint32_t s, int M) {
  uint32_t r = 0;
  int k = 0;
  for (int b = 0; b < M; ++b)
    if (s >> b & 1) {
      ++k;
      r += (uint32_t)binom(b, k);
    }
  return r;
}

struct Z {
  double x, y;
};

// The quad-split pair update of the kernels (lane q: own component x1, partner
// component x2, out = x1 c + x2 s with s = -t or t by parity and component).
void pair_update(Z& l, Z& r, double c, double t, uint32_t par) {
  const double s0 = (par ^ 1u) ? -t : t, s1 = par ? -t : t;
  volatile double a = l.x * c, b = r.y * s0;
  const double lx = a + b;
  a = l.y * c;
  b = r.x * s1;
  const double ly = a + b;
  a = r.x * c;
  b = l.y * s0;
  const double rx = a + b;
  a = r.y * c;
  b = l.x * s1;
  const double ry = a + b;
  l = {lx, ly};
  r = {rx, ry};
}

}  // namespace

// stats[0..3]: scheduled passes, windows, words per warp program, largest
// number of quads any CTA runs at one level.
extern "C" int mix_units_check(unsigned M, unsigned na, unsigned nb, const qpe_term* const* terms, const size_t* n,
                               unsigned order, unsigned K, unsigned wpc, unsigned stage, unsigned max_window,
                               unsigned* stats) {
  TermArrays T;
  for (int k = 0; k < 5; ++k) {
    T.t[k] = terms[k];
    T.n[k] = n[k];
  }
  HostProgram hp;
  build_program(hp, M, na, nb, T, order, 1);
  std::vector<uint32_t> pool(hp.pool_words, 0u);
  for (const AxisTable& tb : hp.tables) {
    if (tb.kind != AX_CA) continue;
    const int p = tb.o[0], r = tb.o[1];
    uint32_t j = 0;
    for (uint32_t s = 0; s < (1u << M); ++s) {
      if (__builtin_popcount(s) != tb.weight || !(s >> r & 1) || (s >> p & 1)) continue;
      const int lo = p < r ? p : r, hi = p < r ? r : p;
      const uint32_t between = s & ((1u << hi) - 1) & ~((1u << (lo + 1)) - 1);
      pool[tb.offset + 2 * j] = colex_rank(s, M) | ((uint32_t)(__builtin_popcount(between) & 1) << 31);
      pool[tb.offset + 2 * j + 1] = colex_rank(s ^ (1u << r) ^ (1u << p), M);
      ++j;
    }
    if (j != tb.count) return -1;
  }
  MixUnits mu;
  build_mix_units(hp, pool.data(), K, wpc, stage, max_window, mu);
  stats[0] = mu.scheduled;
  stats[1] = mu.windows;
  stats[2] = mu.wp_words;
  stats[3] = 0;
  const uint32_t Ca = (uint32_t)hp.Ca, Cb = (uint32_t)hp.Cb, groups = wpc / 3;
  int bad = 0;
  std::mt19937_64 rng(7);
  std::uniform_real_distribution<double> U(-1, 1);
  std::vector<Z> A((size_t)Ca * Cb), B;
  for (Z& v : A) v = {U(rng), U(rng)};
  B = A;
  for (size_t pi = 0; pi < hp.passes.size(); ++pi) {
    const uint32_t m = mu.pass_slot[pi];
    if (m == kMixNoSchedule) continue;
    const uint32_t span = (m >> 20) & 0xffu, slot = m & 0xfffffu;
    uint32_t levels = 0;
    for (uint32_t q = 0; q < span; ++q) {
      if (pi + q >= hp.passes.size() || mu.pass_slot[pi + q] != m) return bad + 1;
      const Pass& ps = hp.passes[pi + q];
      levels += ps.op1 - ps.op0;
      for (uint32_t tl = 0; tl < ps.mixcount; ++tl) {
        const uint32_t w0 = pool[ps.mixtab + 2 * tl], b10 = pool[ps.mixtab + 2 * tl + 1];
        const uint32_t b01 = w0 & 0x7fffffffu, parb = w0 >> 31;
        for (uint32_t k = ps.op0; k < ps.op1; ++k) {
          const DevOp& d = hp.ops[k];
          for (uint32_t j = 0; j < d.count; ++j) {
            const uint32_t e0 = pool[d.tab + 2 * j], a10 = pool[d.tab + 2 * j + 1];
            pair_update(A[(size_t)(e0 & 0x7fffffffu) * Cb + b01], A[(size_t)a10 * Cb + b10], d.c0, d.c1,
                        (e0 >> 31) ^ parb);
          }
        }
      }
    }
    const uint32_t op0 = hp.passes[pi].op0;
    const uint32_t* blk = mu.words.data() + (size_t)slot * K * wpc * mu.wp_words;
    auto W = [&](uint32_t r, uint32_t w) { return blk + ((size_t)r * wpc + w) * mu.wp_words; };
    auto team_of = [&](uint32_t r, uint32_t w) {
      return ((W(r, w)[0] >> 7) & 3u) > 1 ? r * wpc + (w / 3) * 3 : r * wpc + w;
    };
    std::vector<Z> st((size_t)K * groups * stage, Z{0, 0});
    std::vector<int> owner(st.size(), -1);
    std::set<uint64_t> gathered;
    for (uint32_t r = 0; r < K; ++r)
      for (uint32_t g = 0; g < groups; ++g) {
        const uint32_t h0 = W(r, 3 * g)[0], tw0 = (h0 >> 7) & 3u;
        for (uint32_t i = 0; i < 3; ++i) {
          const uint32_t h = W(r, 3 * g + i)[0], tw = (h >> 7) & 3u;
          if (tw0 > 1 && i < tw0) bad += tw != tw0 || ((h >> 9) & 0xffu) != ((h0 >> 9) & 0xffu);
          else bad += tw > 1;
          if (tw) bad += ((h >> 9) & 0xffu) != levels || W(r, 3 * g + i)[1] != op0;
          bad += (h & 127u) > kMixWarpAmps || (!tw && (h & 127u));
        }
      }
    for (uint32_t r = 0; r < K; ++r)
      for (uint32_t w = 0; w < wpc; ++w) {
        const uint32_t* p = W(r, w);
        const uint32_t nel = ((p[0] >> 7) & 3u) ? p[0] & 127u : 0u;
        for (uint32_t l = 0; l < nel; ++l) {
          const uint32_t gw = p[kMixWpHeader + l], row = gw & 2047u, col = (gw >> 11) & 2047u, si = gw >> 22;
          if (row >= Ca || col >= Cb || si >= stage) {
            ++bad;
            continue;
          }
          bad += !gathered.insert((uint64_t)row * Cb + col).second;
          const size_t gi = ((size_t)r * groups + w / 3) * stage + si;
          bad += owner[gi] >= 0;
          owner[gi] = (int)team_of(r, w);
          st[gi] = B[(size_t)row * Cb + col];
        }
      }
    for (uint32_t lv = 0; lv < levels; ++lv) {
      const DevOp& d = hp.ops[op0 + lv];
      for (uint32_t r = 0; r < K; ++r) {
        uint32_t quads = 0;
        for (uint32_t w = 0; w < wpc; ++w) {
          const uint32_t* p = W(r, w);
          if (!((p[0] >> 7) & 3u)) continue;
          const size_t base = ((size_t)r * groups + w / 3) * stage;
          for (uint32_t u = 0; u < 8; ++u) {
            const uint32_t uw = p[kMixWpHeader + kMixWarpAmps + 8 * lv + u];
            if (!((uw >> 21) & 1u)) continue;
            ++quads;
            const uint32_t li = uw & 1023u, ri = (uw >> 10) & 1023u;
            if (li >= stage || ri >= stage || owner[base + li] != (int)team_of(r, w) ||
                owner[base + ri] != (int)team_of(r, w)) {
              ++bad;
              continue;
            }
            pair_update(st[base + li], st[base + ri], d.c0, d.c1, (uw >> 20) & 1u);
          }
        }
        if (quads > stats[3]) stats[3] = quads;
      }
    }
    for (uint32_t r = 0; r < K; ++r)
      for (uint32_t w = 0; w < wpc; ++w) {
        const uint32_t* p = W(r, w);
        const uint32_t nel = ((p[0] >> 7) & 3u) ? p[0] & 127u : 0u;
        for (uint32_t l = 0; l < nel; ++l) {
          const uint32_t gw = p[kMixWpHeader + l];
          if ((gw & 2047u) < Ca && ((gw >> 11) & 2047u) < Cb && (gw >> 22) < stage)
            B[(size_t)(gw & 2047u) * Cb + ((gw >> 11) & 2047u)] = st[((size_t)r * groups + w / 3) * stage + (gw >> 22)];
        }
      }
    if (std::memcmp(A.data(), B.data(), A.size() * sizeof(Z)) != 0) {
      ++bad;
      B = A;
    }
    pi += span - 1;
  }
  return bad;
}
