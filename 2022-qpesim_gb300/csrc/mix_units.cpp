// mix_units.cpp - the host scheduler of the column-pair passes' update units
// (mix_units.h).
#include "mix_units.h"

#include <algorithm>
#include <numeric>

namespace qpe {

namespace {

constexpr uint32_t kQuads = 8;         // quads of lanes per warp
constexpr uint32_t kLanes = kMixWarpAmps;  // amplitudes a warp gathers (two per lane)
constexpr uint32_t kMaxTeam = 3;       // warps of a three-warp group
constexpr uint32_t kIdxLimit = 1024;   // stage indices are 10-bit
constexpr uint32_t kLineLimit = 2048;  // rows and columns are 11-bit

struct Upd {
  uint32_t l, r, par;  // unit-local amplitude indices, parity of the update
};

// One connected component of a window's pairings: its amplitudes (row * Cb +
// col) and its updates per level.
struct Comp {
  std::vector<uint32_t> nodes;
  std::vector<std::vector<Upd>> lev;
  uint32_t maxper = 0;
};

// Work placed on warps: one unit on a team of `tw` warps, or several small units
// on one warp (tw = 1).
struct Team {
  uint32_t tw = 1;
  std::vector<uint32_t> units;
  uint32_t quads = 0, elems = 0;  // most update slots at one level, amplitudes
  std::vector<uint32_t> used;     // update slots per level (packs of small units)
};

struct UnionFind {
  std::vector<uint32_t> p;
  explicit UnionFind(size_t n) : p(n) { std::iota(p.begin(), p.end(), 0u); }
  uint32_t find(uint32_t x) {
    while (p[x] != x) {
      p[x] = p[p[x]];
      x = p[x];
    }
    return x;
  }
  void join(uint32_t a, uint32_t b) {
    a = find(a);
    b = find(b);
    if (a != b) p[std::max(a, b)] = std::min(a, b);
  }
};

// Visits every update of passes [w0, w1) in order: f(level, left amplitude,
// right amplitude, parity). False if a term is not an inline pair term or an
// index is out of range.
template <class F>
bool for_each_update(const HostProgram& hp, const uint32_t* pool, size_t w0, size_t w1, F f) {
  const uint32_t Ca = (uint32_t)hp.Ca, Cb = (uint32_t)hp.Cb;
  uint32_t lv = 0;
  for (size_t pi = w0; pi < w1; ++pi) {
    const Pass& ps = hp.passes[pi];
    for (uint32_t k = ps.op0; k < ps.op1; ++k, ++lv) {
      const DevOp& d = hp.ops[k];
      if (d.kind != OPK_PAIR || d.gen != OP_INLINE) return false;
      for (uint32_t t = 0; t < ps.mixcount; ++t) {
        const uint32_t pw = pool[ps.mixtab + 2 * t], b10 = pool[ps.mixtab + 2 * t + 1];
        const uint32_t b01 = pw & 0x7fffffffu;
        if (b01 >= Cb || b10 >= Cb) return false;
        for (uint32_t j = 0; j < d.count; ++j) {
          const uint32_t w = pool[d.tab + 2 * j], a01 = w & 0x7fffffffu, a10 = pool[d.tab + 2 * j + 1];
          if (a01 >= Ca || a10 >= Ca) return false;
          f(lv, a01 * Cb + b01, a10 * Cb + b10, (w >> 31) ^ (pw >> 31));
        }
      }
    }
  }
  return true;
}

// The components of the window [w0, w1); false if it cannot be scheduled.
bool window_components(const HostProgram& hp, const uint32_t* pool, size_t w0, size_t w1, uint32_t levels,
                       std::vector<Comp>& comps) {
  UnionFind uf((size_t)hp.Ca * hp.Cb);
  if (!for_each_update(hp, pool, w0, w1, [&](uint32_t, uint32_t x, uint32_t y, uint32_t) { uf.join(x, y); }))
    return false;
  std::vector<int> cid(uf.p.size(), -1), lidx(uf.p.size(), -1);
  comps.clear();
  for_each_update(hp, pool, w0, w1, [&](uint32_t lv, uint32_t x, uint32_t y, uint32_t par) {
    const uint32_t root = uf.find(x);
    if (cid[root] < 0) {
      cid[root] = (int)comps.size();
      comps.emplace_back();
      comps.back().lev.resize(levels);
    }
    Comp& c = comps[cid[root]];
    for (uint32_t node : {x, y})
      if (lidx[node] < 0) {
        lidx[node] = (int)c.nodes.size();
        c.nodes.push_back(node);
      }
    c.lev[lv].push_back({(uint32_t)lidx[x], (uint32_t)lidx[y], par});
  });
  for (Comp& c : comps)
    for (const auto& l : c.lev) c.maxper = std::max<uint32_t>(c.maxper, (uint32_t)l.size());
  return true;
}

// Team warps a unit of component c needs (0: too large for a group).
uint32_t team_warps(const Comp& c) {
  const uint32_t tw = std::max((c.maxper + kQuads - 1) / kQuads, ((uint32_t)c.nodes.size() + kLanes - 1) / kLanes);
  return tw <= kMaxTeam ? std::max(tw, 1u) : 0u;
}

// Places the units of one window and writes its warp programs into `block`
// (K * wpc programs of wp_words words). False if some unit does not fit.
bool place_window(const HostProgram& hp, const std::vector<Comp>& comps, uint32_t op0, uint32_t levels, uint32_t K,
                  uint32_t wpc, uint32_t stage_elems, uint32_t wp_words, uint32_t* block) {
  const uint32_t groups = wpc / kMaxTeam;
  std::vector<Team> teams;
  // large units: one team each; small ones packed first-fit, largest first
  std::vector<uint32_t> small;
  for (uint32_t c = 0; c < comps.size(); ++c) {
    const uint32_t tw = team_warps(comps[c]);
    if (tw == 0) return false;
    if (tw == 1) {
      small.push_back(c);
      continue;
    }
    Team tm;
    tm.tw = tw;
    tm.units.push_back(c);
    tm.quads = comps[c].maxper;
    tm.elems = (uint32_t)comps[c].nodes.size();
    teams.push_back(tm);
  }
  std::stable_sort(teams.begin(), teams.end(), [](const Team& a, const Team& b) { return a.quads > b.quads; });
  auto total = [&](uint32_t c) {
    size_t t = 0;
    for (const auto& l : comps[c].lev) t += l.size();
    return t;
  };
  std::stable_sort(small.begin(), small.end(), [&](uint32_t a, uint32_t b) { return total(a) > total(b); });
  // A warp's quads are reassigned at every level, so small units share a warp
  // as long as their updates at each level fit its 8 quads (and their
  // amplitudes its 32 lanes): fewer warps, and fewer FP64 instructions per level
  // on each SM sub-partition.
  std::vector<Team> packs;
  for (uint32_t c : small) {
    const Comp& cc = comps[c];
    const uint32_t e = (uint32_t)cc.nodes.size();
    Team* fit = nullptr;
    for (Team& pk : packs) {
      if (pk.elems + e > kLanes) continue;
      bool ok = true;
      for (uint32_t k = 0; k < levels && ok; ++k) ok = pk.used[k] + cc.lev[k].size() <= kQuads;
      if (ok) {
        fit = &pk;
        break;
      }
    }
    if (!fit) {
      packs.emplace_back();
      fit = &packs.back();
      fit->used.assign(levels, 0);
    }
    fit->units.push_back(c);
    fit->elems += e;
    for (uint32_t k = 0; k < levels; ++k) {
      fit->used[k] += (uint32_t)cc.lev[k].size();
      fit->quads = std::max(fit->quads, fit->used[k]);
    }
  }
  teams.insert(teams.end(), packs.begin(), packs.end());
  // Place each team where it adds least to the most warps on one SM
  // sub-partition of a CTA (warp w runs on sub-partition w % 4; an FP64
  // instruction holds its sub-partition's unit for about 62 cycles, so two warps
  // there double a level's FP64 time), then where the CTA has the fewest update
  // slots per level. A team of two or three warps takes warps 0 .. tw - 1 of an
  // empty group (it synchronises by the group's named barrier); a single warp
  // any free warp of a group; the group's stage must have room for its amplitudes.
  std::vector<uint32_t> load(K, 0), gmask((size_t)K * groups, 0), gstage((size_t)K * groups, 0);
  std::vector<uint32_t> sub((size_t)K * 4, 0);
  std::fill(block, block + (size_t)K * wpc * wp_words, 0u);
  const uint32_t Cb = (uint32_t)hp.Cb;
  for (const Team& tm : teams) {
    int best_cta = -1;
    uint32_t best_w0 = 0, best_score0 = ~0u, best_score1 = ~0u;
    for (uint32_t r = 0; r < K; ++r)
      for (uint32_t g = 0; g < groups; ++g) {
        const size_t gi = (size_t)r * groups + g;
        if (gstage[gi] + tm.elems > stage_elems) continue;
        for (uint32_t i = 0; i < (tm.tw > 1 ? 1u : kMaxTeam); ++i) {
          const uint32_t bits = tm.tw > 1 ? (1u << tm.tw) - 1 : 1u << i;
          if (gmask[gi] & (tm.tw > 1 ? 7u : bits)) continue;
          uint32_t worst = 0;
          for (uint32_t s4 = 0; s4 < 4; ++s4) {
            uint32_t c = sub[(size_t)r * 4 + s4];
            for (uint32_t w = 0; w < kMaxTeam; ++w)
              if ((bits >> w & 1u) && (g * kMaxTeam + w) % 4 == s4) ++c;
            worst = std::max(worst, c);
          }
          const uint32_t score1 = load[r] + tm.quads;
          if (worst < best_score0 || (worst == best_score0 && score1 < best_score1)) {
            best_score0 = worst;
            best_score1 = score1;
            best_cta = (int)r;
            best_w0 = g * kMaxTeam + (tm.tw > 1 ? 0u : i);
          }
        }
      }
    if (best_cta < 0) return false;
    const uint32_t g = best_w0 / kMaxTeam;
    const size_t gi = (size_t)best_cta * groups + g;
    const uint32_t w0 = best_w0;
    const uint32_t ebase = gstage[gi];
    for (uint32_t w = 0; w < tm.tw; ++w) {
      gmask[gi] |= 1u << (w0 + w - g * kMaxTeam);
      ++sub[(size_t)best_cta * 4 + (w0 + w) % 4];
    }
    gstage[gi] += tm.elems;
    load[best_cta] += tm.quads;
    if (ebase + tm.elems > kIdxLimit) return false;
    // amplitudes: element i of the team goes to warp i / 32, lane i % 32, and to
    // stage index ebase + i of the group; updates of level k: quad slot j goes to
    // warp j / 8, quad j % 8
    uint32_t* wp[kMaxTeam];
    for (uint32_t w = 0; w < tm.tw; ++w) {
      wp[w] = block + ((size_t)best_cta * wpc + w0 + w) * wp_words;
      wp[w][0] = (tm.tw << 7) | (levels << 9);
      wp[w][1] = op0;
    }
    uint32_t e0 = 0;
    std::vector<uint32_t> q0(levels, 0);  // update slots taken at each level
    for (uint32_t ci : tm.units) {
      const Comp& c = comps[ci];
      for (uint32_t i = 0; i < c.nodes.size(); ++i) {
        const uint32_t row = c.nodes[i] / Cb, col = c.nodes[i] % Cb, e = e0 + i;
        uint32_t* w = wp[e / kLanes];
        w[kMixWpHeader + e % kLanes] = row | (col << 11) | ((ebase + e) << 22);
        w[0] = (w[0] & ~127u) | ((w[0] & 127u) + 1);
      }
      for (uint32_t k = 0; k < levels; ++k)
        for (uint32_t j = 0; j < c.lev[k].size(); ++j) {
          const Upd& up = c.lev[k][j];
          const uint32_t slot = q0[k]++;
          wp[slot / kQuads][kMixWpHeader + kLanes + kQuads * k + slot % kQuads] =
              (ebase + e0 + up.l) | ((ebase + e0 + up.r) << 10) | (up.par << 20) | (1u << 21);
        }
      e0 += (uint32_t)c.nodes.size();
    }
  }
  return true;
}

}  // namespace

uint32_t mix_wp_words(const HostProgram&) { return (kMixWpHeader + kLanes + kQuads * kMixMaxLevels + 3) & ~3u; }

bool build_mix_units(const HostProgram& hp, const uint32_t* pool, uint32_t K, uint32_t warps_per_cta,
                     uint32_t stage_elems, uint32_t max_window, MixUnits& out) {
  out = MixUnits{};
  if (hp.Ca >= kLineLimit || hp.Cb >= kLineLimit || K == 0 || warps_per_cta < kMaxTeam || max_window == 0)
    return false;
  if (hp.Ca * hp.Cb > (1u << 22)) return false;  // the union-find runs over the block's amplitudes
  const uint32_t full = mix_wp_words(hp);
  const size_t block = (size_t)K * warps_per_cta * full;
  out.warps_per_cta = warps_per_cta;
  out.cluster = K;
  out.pass_slot.assign(hp.passes.size(), kMixNoSchedule);
  struct Window {
    size_t w0, w1;
    uint32_t levels;
    std::vector<uint32_t> words;  // K * wpc programs of `full` words
  };
  std::vector<Window> wins;
  std::vector<Comp> comps;
  std::vector<uint32_t> trial(block);
  auto mixable = [&](size_t pi) {
    const Pass& p = hp.passes[pi];
    return p.type == PASS_MIX && p.op1 > p.op0 && p.mixcount > 0;
  };
  size_t pi = 0;
  while (pi < hp.passes.size()) {
    if (!mixable(pi)) {
      ++pi;
      continue;
    }
    // grow [pi, end) one pass at a time while the window still schedules
    Window best{pi, pi, 0, {}};
    uint32_t levels = 0;
    for (size_t end = pi + 1; end <= hp.passes.size() && end - pi <= max_window; ++end) {
      if (!mixable(end - 1)) break;
      levels += hp.passes[end - 1].op1 - hp.passes[end - 1].op0;
      if (levels > kMixMaxLevels) break;
      if (!window_components(hp, pool, pi, end, levels, comps)) break;
      if (!place_window(hp, comps, hp.passes[pi].op0, levels, K, warps_per_cta, stage_elems, full, trial.data()))
        break;
      best.w1 = end;
      best.levels = levels;
      best.words = trial;
    }
    if (best.w1 == pi) {
      ++pi;  // this pass runs by tiles
      continue;
    }
    pi = best.w1;
    wins.push_back(std::move(best));
  }
  if (wins.empty()) return false;
  // the programs at the size the longest window needs
  uint32_t lmax = 1;
  for (const Window& w : wins) lmax = std::max(lmax, w.levels);
  out.wp_words = (kMixWpHeader + kLanes + kQuads * lmax + 3) & ~3u;
  const size_t progs = (size_t)K * warps_per_cta;
  out.words.assign(wins.size() * progs * out.wp_words, 0u);
  for (size_t wi = 0; wi < wins.size(); ++wi) {
    for (size_t p = 0; p < progs; ++p)
      std::copy_n(wins[wi].words.data() + p * full, out.wp_words, out.words.data() + (wi * progs + p) * out.wp_words);
    const uint32_t span = (uint32_t)(wins[wi].w1 - wins[wi].w0);
    for (size_t q = wins[wi].w0; q < wins[wi].w1; ++q) out.pass_slot[q] = (uint32_t)wi | (span << 20);
    out.scheduled += span;
  }
  out.windows = (uint32_t)wins.size();
  return true;
}

bool build_line_units(const HostProgram& hp, const uint32_t* pool, const uint32_t* strA, const uint32_t* strB,
                      uint32_t K, uint32_t warps_per_cta, uint32_t rows_per_cta, uint32_t replicas,
                      uint32_t stage_elems, LineUnits& out) {
  out = LineUnits{};
  out.replicas = replicas = std::max(replicas, 1u);
  out.pass_slot.assign(hp.passes.size(), kMixNoSchedule);
  const uint32_t groups = warps_per_cta / kMaxTeam, Ca = (uint32_t)hp.Ca, Cb = (uint32_t)hp.Cb;
  if (K < 2 || groups == 0 || Ca >= kLineLimit || Cb >= kLineLimit) return false;
  const size_t block = (size_t)replicas * K * warps_per_cta;
  constexpr uint32_t kLevelWords = 1 + kQuads, kTeam = kMaxTeam;
  constexpr uint32_t kPairCap = kTeam * kQuads, kDiagCap = kTeam * 2 * kQuads;  // updates per level
  for (size_t pi = 0; pi < hp.passes.size(); ++pi) {
    const Pass& ps = hp.passes[pi];
    if (ps.type == PASS_MIX || ps.op1 <= ps.op0) continue;
    const bool col = ps.type == PASS_COL;
    const uint32_t lines = col ? Cb : Ca, L = col ? Ca : Cb;
    if (L > kTeam * kLanes || L > stage_elems || L > kIdxLimit) continue;
    bool ok = true;
    for (uint32_t k = ps.op0; k < ps.op1 && ok; ++k) ok = hp.ops[k].gen == OP_INLINE;
    if (!ok) continue;
    std::vector<uint32_t> offs(block, kMixNoSchedule);
    std::vector<uint32_t> words;
    const size_t base = out.words.size();
    for (uint32_t ln = 0; ln < lines && ok; ++ln) {
      // the line's replica, CTA and group
      uint32_t r, cta, g;
      if (col) {
        r = ln % replicas;
        const uint32_t j = ln / replicas;
        cta = j % K;
        g = j / K;
      } else {
        cta = ln / rows_per_cta;
        const uint32_t t = ln - cta * rows_per_cta;
        r = t % replicas;
        g = t / replicas;
      }
      if (g >= groups || cta >= K) {
        ok = false;
        break;
      }
      const uint32_t lstr = col ? strB[ln] : strA[ln];
      // levels: (op word, update slots)
      std::vector<uint32_t> lev;  // kTeam * kLevelWords words per level: warp w's op word and 8 update words
      auto new_level = [&](uint32_t opw) {
        const size_t at = lev.size();
        lev.resize(at + kTeam * kLevelWords, 0u);
        for (uint32_t w = 0; w < kTeam; ++w) lev[at + w * kLevelWords] = opw;
        return at;
      };
      for (uint32_t k = ps.op0; k < ps.op1; ++k) {
        const DevOp& d = hp.ops[k];
        uint32_t m = 0;
        if (d.ncond > 0) m |= 1u << d.cb0;
        if (d.ncond > 1) m |= 1u << d.cb1;
        if ((lstr & m) != m) continue;  // the term does not act on this line
        const uint32_t count = d.kind == OPK_DIAG_ALL ? L : d.count;
        if (count == 0) continue;
        const uint32_t op = k - ps.op0;  // index within the pass: the kernel reverses it
        if (d.kind == OPK_PAIR) {
          for (uint32_t j0 = 0; j0 < count; j0 += kPairCap) {
            const size_t at = new_level(op);
            for (uint32_t j = j0; j < std::min(count, j0 + kPairCap); ++j) {
              const uint32_t w0 = pool[d.tab + 2 * j], a01 = w0 & 0x7fffffffu, a10 = pool[d.tab + 2 * j + 1];
              if (a01 >= L || a10 >= L) ok = false;
              const uint32_t s = j - j0;
              lev[at + (s / kQuads) * kLevelWords + 1 + s % kQuads] =
                  a01 | (a10 << 10) | ((w0 >> 31) << 20) | (1u << 21);
            }
          }
        } else {
          for (uint32_t j0 = 0; j0 < count; j0 += kDiagCap) {
            const size_t at = new_level(op | 0x80000000u);
            for (uint32_t j = j0; j < std::min(count, j0 + kDiagCap); ++j) {
              const uint32_t e = d.kind == OPK_DIAG_LIST ? pool[d.tab + j] : j;
              if (e >= L) ok = false;
              const uint32_t s = j - j0, w = s / (2 * kQuads), u = (s % (2 * kQuads)) / 2, half = s & 1u;
              uint32_t& word = lev[at + w * kLevelWords + 1 + u];
              word |= (e << (10 * half)) | (1u << (20 + half));
            }
          }
        }
      }
      const uint32_t nlev = (uint32_t)(lev.size() / (kTeam * kLevelWords));
      // the team's three programs
      for (uint32_t w = 0; w < kTeam; ++w) {
        const uint32_t off = (uint32_t)(base + words.size());
        offs[((size_t)r * K + cta) * warps_per_cta + g * kTeam + w] = off;
        const uint32_t e0 = w * kLanes, e1 = std::min(L, e0 + kLanes), nel = e1 > e0 ? e1 - e0 : 0u;
        std::vector<uint32_t> prog(kMixWpHeader + kLanes + (size_t)nlev * kLevelWords, 0u);
        prog[0] = nel | (kTeam << 7);
        prog[1] = nlev;
        for (uint32_t e = e0; e < e1; ++e) {
          const uint32_t row = col ? e : ln, cc = col ? ln : e;
          prog[kMixWpHeader + (e - e0)] = row | (cc << 11) | (e << 22);
        }
        for (uint32_t lv = 0; lv < nlev; ++lv)
          std::copy_n(lev.data() + ((size_t)lv * kTeam + w) * kLevelWords, kLevelWords,
                      prog.data() + kMixWpHeader + kLanes + (size_t)lv * kLevelWords);
        // pad to 16 bytes
        prog.resize((prog.size() + 3) & ~(size_t)3, 0u);
        words.insert(words.end(), prog.begin(), prog.end());
      }
    }
    if (!ok) continue;
    out.pass_slot[pi] = out.passes++;
    out.offs.insert(out.offs.end(), offs.begin(), offs.end());
    out.words.insert(out.words.end(), words.begin(), words.end());
  }
  return out.passes > 0;
}

}  // namespace qpe
