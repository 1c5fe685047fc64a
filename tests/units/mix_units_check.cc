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

// Per-line programs of the row and column passes: every scheduled pass is run
// both the line runner's way (per line, each term whose condition orbitals the
// line's string has, in order: pair updates as above, diagonal updates v (c0 +
// i c1) split as the kernels split them) and the way k_resident_lean runs the
// programs (gather per team into its group's stage, level by level, scatter),
// on a random complex128 block; returns the number of differences and broken
// invariants (line placement by replica, team layout, bounds, one program per
// line, op words inside the pass). stats: passes with programs, levels in all.
extern "C" int line_units_check(unsigned M, unsigned na, unsigned nb, const qpe_term* const* terms, const size_t* n,
                                unsigned order, unsigned K, unsigned wpc, unsigned stage, unsigned replicas,
                                unsigned* stats) {
  TermArrays T;
  for (int k = 0; k < 5; ++k) {
    T.t[k] = terms[k];
    T.n[k] = n[k];
  }
  HostProgram hp;
  build_program(hp, M, na, nb, T, order, 1);
  const uint32_t Ca = (uint32_t)hp.Ca, Cb = (uint32_t)hp.Cb;
  // line strings by colex rank
  std::vector<uint32_t> strA(Ca), strB(Cb);
  for (uint32_t s = 0; s < (1u << M); ++s) {
    if ((uint32_t)__builtin_popcount(s) == na) strA[colex_rank(s, M)] = s;
    if ((uint32_t)__builtin_popcount(s) == nb) strB[colex_rank(s, M)] = s;
  }
  // every table: lists of strings with the listed orbitals occupied, pairs of
  // strings that move the 10 side's electrons to the 01 side's orbitals
  std::vector<uint32_t> pool(hp.pool_words, 0u);
  for (const AxisTable& tb : hp.tables) {
    uint32_t need = 0, empty = 0, moveA = 0, moveB = 0;  // 01 side: need occupied, empty empty
    bool pairs = true;
    switch (tb.kind) {
      case AX_N: need = 1u << tb.o[0]; pairs = false; break;
      case AX_NN: need = (1u << tb.o[0]) | (1u << tb.o[1]); pairs = false; break;
      case AX_CA: need = 1u << tb.o[1]; empty = 1u << tb.o[0]; break;
      case AX_CNA: need = (1u << tb.o[1]) | (1u << tb.o[2]); empty = 1u << tb.o[0]; break;
      case AX_CCAA: need = (1u << tb.o[2]) | (1u << tb.o[3]); empty = (1u << tb.o[0]) | (1u << tb.o[1]); break;
    }
    moveA = tb.kind == AX_CNA ? (1u << tb.o[2]) | (1u << tb.o[0]) : need | empty;
    (void)moveB;
    uint32_t j = 0;
    const std::vector<uint32_t>& byrank = tb.weight == na ? strA : strB;  // colex order
    for (uint32_t s : byrank) {
      if ((s & need) != need || (s & empty)) continue;
      if (pairs) {
        pool[tb.offset + 2 * j] = colex_rank(s, M) | ((uint32_t)(__builtin_popcount(s) & 1) << 31);
        pool[tb.offset + 2 * j + 1] = colex_rank(s ^ moveA, M);
      } else {
        pool[tb.offset + j] = colex_rank(s, M);
      }
      ++j;
    }
    if (j != tb.count) return -1;
  }
  const uint32_t Rk = (Ca + K - 1) / K, groups = wpc / 3;
  LineUnits lu;
  build_line_units(hp, pool.data(), strA.data(), strB.data(), K, wpc, Rk, replicas, stage, lu);
  stats[0] = lu.passes;
  stats[1] = 0;
  int bad = 0;
  std::mt19937_64 rng(11);
  std::uniform_real_distribution<double> U(-1, 1);
  std::vector<Z> A((size_t)Ca * Cb), B;
  for (Z& v : A) v = {U(rng), U(rng)};
  B = A;
  auto diag_update = [](Z& v, double c, double t) {
    volatile double a = v.x * c, b = v.y * -t;
    const double x = a + b;
    a = v.y * c;
    b = v.x * t;
    v = {x, a + b};
  };
  for (size_t pi = 0; pi < hp.passes.size(); ++pi) {
    const uint32_t slot = lu.pass_slot[pi];
    if (slot == kMixNoSchedule) continue;
    const Pass& ps = hp.passes[pi];
    const bool col = ps.type == PASS_COL;
    if (ps.type == PASS_MIX) return bad + 1000;
    const uint32_t lines = col ? Cb : Ca, L = col ? Ca : Cb;
    auto amp = [&](std::vector<Z>& X, uint32_t ln, uint32_t e) -> Z& {
      return col ? X[(size_t)e * Cb + ln] : X[(size_t)ln * Cb + e];
    };
    // the line runner's way
    for (uint32_t ln = 0; ln < lines; ++ln) {
      const uint32_t lstr = col ? strB[ln] : strA[ln];
      for (uint32_t k = ps.op0; k < ps.op1; ++k) {
        const DevOp& d = hp.ops[k];
        uint32_t m = 0;
        if (d.ncond > 0) m |= 1u << d.cb0;
        if (d.ncond > 1) m |= 1u << d.cb1;
        if ((lstr & m) != m) continue;
        const uint32_t count = d.kind == OPK_DIAG_ALL ? L : d.count;
        for (uint32_t j = 0; j < count; ++j) {
          if (d.kind == OPK_PAIR) {
            const uint32_t w0 = pool[d.tab + 2 * j];
            pair_update(amp(A, ln, w0 & 0x7fffffffu), amp(A, ln, pool[d.tab + 2 * j + 1]), d.c0, d.c1, w0 >> 31);
          } else {
            diag_update(amp(A, ln, d.kind == OPK_DIAG_LIST ? pool[d.tab + j] : j), d.c0, d.c1);
          }
        }
      }
    }
    // the programs' way, replica by replica (each replica's lines)
    std::vector<int> seen(lines, 0);
    for (uint32_t r = 0; r < replicas; ++r)
      for (uint32_t cta = 0; cta < K; ++cta)
        for (uint32_t g = 0; g < groups; ++g) {
          const uint32_t* w[3];
          uint32_t offs[3];
          for (uint32_t i = 0; i < 3; ++i) {
            offs[i] = lu.offs[(((size_t)slot * replicas + r) * K + cta) * wpc + 3 * g + i];
            w[i] = offs[i] == kMixNoSchedule ? nullptr : lu.words.data() + offs[i];
          }
          if (!w[0] && !w[1] && !w[2]) continue;
          if (!w[0] || !w[1] || !w[2]) { ++bad; continue; }
          const uint32_t nlev = w[0][1];
          bad += w[1][1] != nlev || w[2][1] != nlev || ((w[0][0] >> 7) & 3u) != 3u;
          std::vector<Z> st(stage, Z{0, 0});
          std::vector<int> mine(stage, 0);
          uint32_t line = ~0u;
          for (uint32_t i = 0; i < 3; ++i) {
            const uint32_t nel = w[i][0] & 127u;
            bad += nel > kMixWarpAmps;
            for (uint32_t l = 0; l < nel; ++l) {
              const uint32_t gw = w[i][kMixWpHeader + l], row = gw & 2047u, cc = (gw >> 11) & 2047u, si = gw >> 22;
              if (row >= Ca || cc >= Cb || si >= stage) { ++bad; continue; }
              const uint32_t ln = col ? cc : row, e = col ? row : cc;
              if (line == ~0u) line = ln;
              bad += ln != line || si != e || mine[si];
              mine[si] = 1;
              st[si] = amp(B, ln, e);
            }
          }
          if (line == ~0u) { ++bad; continue; }
          ++seen[line];
          // placement: the replica that owns the line, the CTA that owns a row
          if (col) bad += line % replicas != r;
          else bad += line / Rk != cta || (line - cta * Rk) % replicas != r;
          stats[1] += nlev;
          for (uint32_t lv = 0; lv < nlev; ++lv) {
            const uint32_t opw = w[0][kMixWpHeader + kMixWarpAmps + 9 * lv];
            const uint32_t op = opw & 0xffffffu;
            if (ps.op0 + op >= ps.op1) { ++bad; continue; }
            const DevOp& d = hp.ops[ps.op0 + op];
            for (uint32_t i = 0; i < 3; ++i) {
              const uint32_t* lvw = w[i] + kMixWpHeader + kMixWarpAmps + 9 * lv;
              bad += lvw[0] != opw;
              for (uint32_t u = 0; u < 8; ++u) {
                const uint32_t uw = lvw[1 + u];
                if (opw >> 31) {
                  for (uint32_t half = 0; half < 2; ++half)
                    if ((uw >> (20 + half)) & 1u) {
                      const uint32_t e = (uw >> (10 * half)) & 1023u;
                      if (e >= stage || !mine[e]) { ++bad; continue; }
                      diag_update(st[e], d.c0, d.c1);
                    }
                } else if ((uw >> 21) & 1u) {
                  const uint32_t li = uw & 1023u, ri = (uw >> 10) & 1023u;
                  if (li >= stage || ri >= stage || !mine[li] || !mine[ri]) { ++bad; continue; }
                  pair_update(st[li], st[ri], d.c0, d.c1, (uw >> 20) & 1u);
                }
              }
            }
          }
          for (uint32_t e = 0; e < stage; ++e)
            if (mine[e]) amp(B, line, e) = st[e];
        }
    for (uint32_t ln = 0; ln < lines; ++ln) bad += seen[ln] != 1;
    if (std::memcmp(A.data(), B.data(), A.size() * sizeof(Z)) != 0) {
      ++bad;
      B = A;
    }
  }
  return bad;
}
