// abi.cu - implementation of the C ABI declared in include/qpe_gb300.h.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "abi_internal.h"
#include "mix_units.h"

namespace qpe {

static thread_local std::string g_last_error;
void set_last_error(const std::string& msg) { g_last_error = msg; }
const std::string& last_error_message() { return g_last_error; }

__global__ void k_set_int(int* p, int v) { *p = v; }

}  // namespace qpe

using namespace qpe;

struct qpe_state {
  qpe_context* ctx = nullptr;
  uint32_t M = 0, na = 0, nb = 0, P = 0;
  int dtype = QPE_C128;
  uint64_t Ca = 0, Cb = 0, ld = 0, N = 0;
  size_t esz = 16;
  DevBuf data, work, dk, partial, probs, tw;
  uint32_t qift_T = 1, qift_grid = 1;
  bool probs_valid = false;
  // Cached one-power graph for the last program evolved on this state.
  uint64_t graph_prog = 0;
  uint32_t graph_exact = 1;
  cudaGraphExec_t graph = nullptr;
  // Resident-kernel descriptor and the autotuned strategy per program.
  DevBuf res_inst;
  uint64_t tuned_prog = 0;
  uint32_t tuned_exact = 1;
  uint32_t tuned_strategy = 0, tuned_cluster = 0, tuned_replicas = 1;
  uint32_t last_strategy = 0, last_cluster = 0, last_replicas = 1;
  // Replica exchange of the lean kernel (ResidentInstance::xbuf, xflag).
  DevBuf xbuf, xflag;
  ~qpe_state() {
    if (graph) cudaGraphExecDestroy(graph);
  }
};

namespace qpe {

static void use_device(qpe_context* ctx) { QPE_CK(cudaSetDevice(ctx->device)); }

static void check_ctx(qpe_context* ctx) {
  if (!ctx) throw Error(QPE_ERR_INVALID, "null context");
  use_device(ctx);
}

void qift_geometry(uint32_t P, uint64_t ld, int dtype, int num_sms, size_t smem_optin, uint32_t& T, uint32_t& grid) {
  const size_t esz = dtype == QPE_C128 ? 16 : 8;
  const size_t row_bytes = ((size_t)1 << P) * esz;
  if (row_bytes > smem_optin) throw Error(QPE_ERR_UNSUPPORTED, "precision too large for the QIFT tile");
  T = 32;
  while (T > 1 && (row_bytes * T > 96 * 1024 || T > ld)) T >>= 1;
  uint64_t tiles = (ld + T - 1) / T;
  uint64_t g = (uint64_t)num_sms * 2;
  if (g > tiles) g = tiles;
  grid = (uint32_t)g;
}

// Twiddles exp(-2 pi i k / N), k < N / 2 (at least one), rounded from long double
// (as the oracle), interleaved (re, im).
std::vector<double> twiddle_table(uint32_t P) {
  const uint64_t N = 1ull << P;
  const uint64_t nh = N / 2 ? N / 2 : 1;
  std::vector<double> twd(2 * nh);
  const long double two_pi = 6.283185307179586476925286766559005768L;
  for (uint64_t k = 0; k < nh; ++k) {
    long double ang = -two_pi * (long double)k / (long double)N;
    twd[2 * k] = (double)cosl(ang);
    twd[2 * k + 1] = (double)sinl(ang);
  }
  return twd;
}

void state_twiddles(uint32_t P, int dtype, DevBuf& tw) {
  const std::vector<double> twd = twiddle_table(P);
  if (dtype == QPE_C128) {
    tw.alloc(twd.size() * sizeof(double));
    QPE_CK(cudaMemcpy(tw.p, twd.data(), twd.size() * sizeof(double), cudaMemcpyHostToDevice));
  } else {
    std::vector<float> twf(twd.begin(), twd.end());
    tw.alloc(twf.size() * sizeof(float));
    QPE_CK(cudaMemcpy(tw.p, twf.data(), twf.size() * sizeof(float), cudaMemcpyHostToDevice));
  }
}

static void state_alloc(qpe_state* st) {
  st->esz = st->dtype == QPE_C128 ? 16 : 8;
  st->N = 1ull << st->P;
  if (st->ld == 0) throw Error(QPE_ERR_INVALID, "empty block");
  st->data.alloc(st->N * st->ld * st->esz);
  st->dk.alloc(sizeof(int));
  st->probs.alloc(st->N * sizeof(double));
  qift_geometry(st->P, st->ld, st->dtype, st->ctx->num_sms, st->ctx->smem_optin, st->qift_T, st->qift_grid);
  st->partial.alloc((size_t)st->qift_grid * st->N * sizeof(double));
  state_twiddles(st->P, st->dtype, st->tw);
  QPE_CK(configure_qift_kernels(st->dtype, qift_smem_bytes(st->P, st->qift_T, st->dtype)));
}

// The image of every MIX pass whose descriptors and tables fit in
// kPassImageMaxBytes: the pass's DevOps with `tab` rewritten to a word offset in
// the image, then each table they use once, every region starting on a 16-byte
// boundary. The descriptors are written here; the tables, which only exist on
// the device, are copied in from the index pool by k_copy_segments.
static void build_pass_images(qpe_program* pr) {
  const HostProgram& hp = pr->hp;
  pr->img_off.assign(hp.passes.size(), 0);
  pr->img_words.assign(hp.passes.size(), 0);
  std::vector<uint32_t> host;
  std::vector<PassImageSeg> segs;
  auto round4 = [](uint64_t w) { return (w + 3) & ~(uint64_t)3; };
  for (size_t pi = 0; pi < hp.passes.size(); ++pi) {
    const Pass& p = hp.passes[pi];
    if (p.type != PASS_MIX || p.op1 <= p.op0) continue;
    const uint32_t n = p.op1 - p.op0;
    std::vector<std::pair<uint32_t, uint32_t>> region;  // (pool word, image word)
    uint64_t words = (uint64_t)n * (sizeof(DevOp) / 4);
    bool ok = true;
    for (uint32_t i = 0; i < n && ok; ++i) {
      const DevOp& d = hp.ops[p.op0 + i];
      if (d.kind != OPK_PAIR) ok = false;
      bool seen = false;
      for (const auto& r : region) seen = seen || r.first == d.tab;
      if (!seen) {
        region.push_back({d.tab, (uint32_t)words});
        words = round4(words + 2ull * d.count);
      }
    }
    words = round4(words);
    if (!ok || words * 4 > kPassImageMaxBytes) continue;
    const size_t base = host.size();
    host.resize(base + words, 0u);
    for (uint32_t i = 0; i < n; ++i) {
      DevOp e = hp.ops[p.op0 + i];
      for (const auto& r : region)
        if (r.first == e.tab) {
          e.tab = r.second;
          break;
        }
      std::memcpy(&host[base + (size_t)i * (sizeof(DevOp) / 4)], &e, sizeof(DevOp));
    }
    for (const auto& r : region) {
      uint32_t count = 0;
      for (uint32_t i = 0; i < n; ++i)
        if (hp.ops[p.op0 + i].tab == r.first) count = hp.ops[p.op0 + i].count;
      segs.push_back({r.first, (uint32_t)(base + r.second), 2 * count});
    }
    pr->img_off[pi] = (uint32_t)base;
    pr->img_words[pi] = (uint32_t)words;
  }
  if (host.empty()) return;
  cudaStream_t s = pr->ctx->stream;
  pr->images.alloc(host.size() * 4);
  QPE_CK(cudaMemcpyAsync(pr->images.p, host.data(), host.size() * 4, cudaMemcpyHostToDevice, s));
  DevBuf dsegs;
  dsegs.alloc(segs.size() * sizeof(PassImageSeg));
  QPE_CK(cudaMemcpyAsync(dsegs.p, segs.data(), segs.size() * sizeof(PassImageSeg), cudaMemcpyHostToDevice, s));
  QPE_CK(launch_copy_segments(pr->pool.as<uint32_t>(), pr->images.as<uint32_t>(), dsegs.as<PassImageSeg>(),
                              (uint32_t)segs.size(), s));
  QPE_CK(cudaStreamSynchronize(s));
}

static void build_device_program(qpe_program* pr) {
  qpe_context* ctx = pr->ctx;
  HostProgram& hp = pr->hp;
  cudaStream_t s = ctx->stream;
  pr->pool.alloc(hp.pool_words * sizeof(uint32_t));
  pr->ops.alloc(hp.ops.size() * sizeof(DevOp));
  pr->coef.alloc(hp.coefs.size() * sizeof(double));
  pr->strA.alloc(hp.Ca * sizeof(uint32_t));
  pr->strB.alloc(hp.Cb * sizeof(uint32_t));
  if (!hp.ops.empty())
    QPE_CK(cudaMemcpyAsync(pr->ops.p, hp.ops.data(), hp.ops.size() * sizeof(DevOp), cudaMemcpyHostToDevice, s));
  if (!hp.coefs.empty())
    QPE_CK(cudaMemcpyAsync(pr->coef.p, hp.coefs.data(), hp.coefs.size() * sizeof(double), cudaMemcpyHostToDevice, s));
  pr->passes.alloc(hp.passes.size() * sizeof(Pass));
  if (!hp.passes.empty())
    QPE_CK(cudaMemcpyAsync(pr->passes.p, hp.passes.data(), hp.passes.size() * sizeof(Pass), cudaMemcpyHostToDevice, s));
  QPE_CK(launch_line_strings(ctx->binom.as<uint64_t>(), hp.M, hp.na, pr->strA.as<uint32_t>(), (uint32_t)hp.Ca, s));
  QPE_CK(launch_line_strings(ctx->binom.as<uint64_t>(), hp.M, hp.nb, pr->strB.as<uint32_t>(), (uint32_t)hp.Cb, s));
  // Index tables: one thread per entry.
  std::vector<uint32_t> start(hp.tables.size() + 1, 0);
  uint64_t total = 0;
  for (size_t i = 0; i < hp.tables.size(); ++i) {
    start[i] = (uint32_t)total;
    total += hp.tables[i].count;
  }
  start[hp.tables.size()] = (uint32_t)total;
  if (!hp.tables.empty()) {
    pr->tabs.alloc(hp.tables.size() * sizeof(AxisTable));
    pr->start.alloc(start.size() * sizeof(uint32_t));
    QPE_CK(cudaMemcpyAsync(pr->tabs.p, hp.tables.data(), hp.tables.size() * sizeof(AxisTable), cudaMemcpyHostToDevice, s));
    QPE_CK(cudaMemcpyAsync(pr->start.p, start.data(), start.size() * sizeof(uint32_t), cudaMemcpyHostToDevice, s));
    QPE_CK(launch_build_tables(ctx->binom.as<uint64_t>(), pr->tabs.as<AxisTable>(), pr->start.as<uint32_t>(),
                               (uint32_t)hp.tables.size(), total, pr->pool.as<uint32_t>(), s));
  }
  QPE_CK(cudaStreamSynchronize(s));
  build_pass_images(pr);
}

// Launch geometry of one pass for elements of esz bytes.
void check_device_error(qpe_context* ctx) {
  int e = 0;
  QPE_CK(cudaMemcpyAsync(&e, ctx->err.p, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
  QPE_CK(cudaStreamSynchronize(ctx->stream));
  if (e) {
    QPE_CK(cudaMemsetAsync(ctx->err.p, 0, sizeof(int), ctx->stream));
    QPE_CK(cudaStreamSynchronize(ctx->stream));
    throw Error(QPE_ERR_TIMEOUT, "a kernel's bounded wait ran out (code " + std::to_string(e) +
                                     ": 2 a tile pass's bulk copies, 4 another replica's exchange); the "
                                     "affected results are invalid");
  }
}

PassLaunch plan_pass_geometry(const qpe_program* pr, size_t esz, size_t smem_optin, const Pass& pass) {
  const HostProgram& hp = pr->hp;
  PassLaunch pl{};
  pl.err = pr->ctx->err.as<int>();
  pl.bulk = (pass.type != PASS_ROW && (hp.Ca * esz) % 16 == 0) ? 1u : 0u;
  const size_t pidx = (size_t)(&pass - hp.passes.data());
  if (pl.bulk && pidx < pr->img_words.size() && pr->img_words[pidx]) {
    pl.img = pr->images.as<uint32_t>() + pr->img_off[pidx];
    pl.img_words = pr->img_words[pidx];
  }

  pl.pool = pr->pool.as<uint32_t>();
  pl.ops = pr->ops.as<DevOp>();
  pl.coef = pr->coef.as<double>();
  pl.strA = pr->strA.as<uint32_t>();
  pl.strB = pr->strB.as<uint32_t>();
  pl.Ca = (uint32_t)hp.Ca;
  pl.Cb = (uint32_t)hp.Cb;
  pl.pass = pass;
  const size_t warp_budget = 24 * 1024;
  uint32_t W = 1;
  if (pass.type == PASS_COL) {
    while (W < 8 && (size_t)hp.Ca * (W * 2) * esz <= warp_budget && (W * 2) * 2 <= hp.Cb) W *= 2;
  }
  pl.W = W;
  const size_t stage = pass_stage_elems(pass, pl.Ca, pl.Cb, W) * esz;
  if (stage > smem_optin) throw Error(QPE_ERR_UNSUPPORTED, "block too large for a shared-memory tile");
  uint32_t wpc = 4;
  while (wpc > 1 && stage * wpc > smem_optin) --wpc;
  uint64_t ntiles = pass.type == PASS_COL ? (hp.Cb + W - 1) / W : (pass.type == PASS_ROW ? hp.Ca : pass.mixcount);
  // Long index tables (tens of entries per lane of a warp): one tile per CTA,
  // whose threads split every term's entries, so a term's chain is short.
  const uint64_t entries = binom((int)hp.M - 2, (int)(pass.type == PASS_ROW ? hp.nb : hp.na) - 1) *
                           (pass.type == PASS_COL ? W : 1);
  pl.cta_tile = entries >= 64 ? kCtaTileThreads : 0u;
  if (pl.cta_tile && pass.type == PASS_COL) {
    // fewer lines per CTA tile while a thread's entries of a term take more than
    // the chunked runner's kPairTrips trips
    const uint64_t e1 = binom((int)hp.M - 2, (int)hp.na - 1);
    while (W > 1 && e1 * W > (uint64_t)kPairTrips * kCtaTileThreads) W /= 2;
    pl.W = W;
    ntiles = (hp.Cb + W - 1) / W;
  }
  if (pl.cta_tile) {
    wpc = pl.cta_tile / 32;
  } else if (esz == 16) {
    // complex128 tiles are bound by the SM's FP64 issue rate: spread the tiles
    // over the SMs first, then stack warps.
    const uint64_t per_sm = (ntiles + pr->ctx->num_sms - 1) / pr->ctx->num_sms;
    wpc = (uint32_t)std::max<uint64_t>(1, std::min<uint64_t>(wpc, per_sm));
  }
  pl.warps_per_cta = wpc;
  const uint32_t slots = pl.cta_tile ? 1u : wpc;
  uint64_t grid = (ntiles + slots - 1) / slots;
  const uint64_t cap = (uint64_t)pr->ctx->num_sms * 8;
  if (grid > cap) grid = cap;
  if (grid < 1) grid = 1;
  pl.grid = (uint32_t)grid;
  if (pl.img && pass_smem_bytes(pl, esz) > smem_optin) {  // the image only where it fits beside the stages
    pl.img = nullptr;
    pl.img_words = 0;
  }
  return pl;
}

static PassLaunch plan_pass(const qpe_program* pr, const qpe_state* st, const Pass& pass) {
  PassLaunch pl = plan_pass_geometry(pr, st->esz, st->ctx->smem_optin, pass);
  pl.work = st->work.p;
  pl.exact = st->dtype == QPE_C128 ? 1u : 0u;
  return pl;
}

// Lines per warp tile W in {1, 2, .., 32}: lane l owns line l % W and walks table
// entries l / W, l / W + 32 / W, ... Minimises (rounds of tiles over the warps) x
// (entries per lane of a typical table); ties go to the smaller stage.
static uint32_t choose_lines(uint64_t lines, uint64_t nwarps, uint64_t entries) {
  uint32_t best = 1;
  uint64_t best_cost = ~0ull;
  for (uint32_t W = 1; W <= 32; W *= 2) {
    const uint64_t tiles = (lines + W - 1) / W;
    const uint64_t rounds = (tiles + nwarps - 1) / nwarps;
    const uint64_t iters = (entries * W + 31) / 32;
    const uint64_t cost = rounds * (iters ? iters : 1);
    if (cost < best_cost) {
      best_cost = cost;
      best = W;
    }
    if (tiles <= 1) break;
  }
  return best;
}

// Geometry of k_resident_lean for cluster size K: three-warp groups (15, 12, 9,
// 6 or 3 warps per CTA), one line or column pair per group tile, a stage of one
// column pair (2 Ca elements) per group when K > 1. With `units` (K > 1) every
// warp also gets a shared-memory slot for its warp program of the column-pair
// update units (mix_units.h).
static bool plan_resident_lean(const qpe_program* pr, const qpe_state* st, uint32_t K, ResidentLaunch& rl,
                               ResidentInstance& ri, bool units = false) {
  const HostProgram& hp = pr->hp;
  const size_t esz = st->esz;
  const uint64_t Ca = hp.Ca, Cb = hp.Cb;
  const uint64_t Rk = (Ca + K - 1) / K;
  const size_t meta = resident_meta_bytes((uint32_t)hp.ops.size(), (uint32_t)hp.pool_words,
                                          (uint32_t)hp.passes.size(), (uint32_t)Ca, (uint32_t)Cb);
  // a group's stage holds one column pair, or with units the amplitudes of its
  // three warps' programs (up to kMixWarpAmps each)
  const uint64_t stage = K > 1 ? std::max<uint64_t>(2 * Ca, units ? 3 * kMixWarpAmps : 0) : 0;
  if (units && K < 2) return false;
  const size_t wp_bytes = units ? (size_t)mix_wp_words(hp) * 4 : 0;
  for (int with_meta = 1; with_meta >= 0; --with_meta)
    for (uint32_t wpc = 15; wpc >= 3; wpc -= 3) {
      // block rows, group stages, the row-pointer table (Ca generic pointers), the
      // warp-program slots, then the metadata
      const size_t head = (size_t)(Rk * Cb * esz + (wpc / 3) * stage * esz);
      const size_t rows =
          ((head + 15) & ~(size_t)15) + ((Ca * sizeof(void*) + 15) & ~(size_t)15) + wpc * wp_bytes;
      const size_t smem = with_meta ? rows + meta : rows;
      if (smem + kResidentStaticSmem > st->ctx->smem_optin) continue;
      ri = ResidentInstance{};
      ri.Ca = (uint32_t)Ca;
      ri.Cb = (uint32_t)Cb;
      ri.rows_per_cta = (uint32_t)Rk;
      ri.Wc = ri.Wr = ri.Wm = 1;
      rl = ResidentLaunch{};
      rl.ninst = 1;
      rl.cluster = K;
      rl.warps_per_cta = wpc;
      rl.stage_elems = (uint32_t)stage;
      rl.meta_smem = (uint32_t)with_meta;
      rl.group = 3;
      rl.smem_bytes = smem < 1024 ? 1024 : smem;
      return true;
    }
  return false;
}

// Geometry of the resident kernel for cluster size K; false if it does not fit.
// mode (ResidentLaunch::group) 0: tiles processed by single warps (k_resident),
// one stage per warp; 1: by four-warp groups (k_resident_group), one stage per
// group; 2: column-pair tiles by four-warp groups, row and column tiles by
// single warps, one stage per warp (a group uses its four warps' stages).
static bool plan_resident(const qpe_program* pr, const qpe_state* st, uint32_t K, ResidentLaunch& rl,
                          ResidentInstance& ri, uint32_t mode = 0) {
  if (mode == 3 || mode == 4) return plan_resident_lean(pr, st, K, rl, ri, mode == 4);
  const bool group = mode == 1;
  const HostProgram& hp = pr->hp;
  const size_t esz = st->esz;
  const uint64_t Ca = hp.Ca, Cb = hp.Cb;
  const uint64_t Rk = (Ca + K - 1) / K;
  uint32_t mixcount = 0;
  for (const Pass& p : hp.passes)
    if (p.type == PASS_MIX) mixcount = std::max(mixcount, p.mixcount);
  const size_t meta = resident_meta_bytes((uint32_t)hp.ops.size(), (uint32_t)hp.pool_words,
                                          (uint32_t)hp.passes.size(), (uint32_t)Ca, (uint32_t)Cb);
  // First choice: the program's metadata staged in shared memory too; then the
  // block (and warp stages) alone.
  for (int with_meta = 1; with_meta >= 0; --with_meta)
  for (uint32_t wpc = 16; wpc >= 4; wpc /= 2) {
    // units that own tiles: warps, or groups of four warps (32 quad slots each)
    const uint32_t units = group ? wpc / 4 : wpc;
    ri = ResidentInstance{};
    ri.Ca = (uint32_t)Ca;
    ri.Cb = (uint32_t)Cb;
    ri.rows_per_cta = (uint32_t)Rk;
    // typical table lengths: CA over alpha (COL / MIX), CA over beta (ROW)
    const uint64_t ea = binom((int)hp.M - 2, (int)hp.na - 1), eb = binom((int)hp.M - 2, (int)hp.nb - 1);
    ri.Wr = choose_lines(Rk, units, eb ? eb : 1);
    ri.Wc = choose_lines(Cb, (uint64_t)K * units, ea ? ea : 1);
    // at most 16 column pairs per tile: a thread's gather column is then fixed
    const uint32_t mix_units = mode == 2 ? wpc / 4 : units;
    ri.Wm = std::min<uint32_t>(16u, choose_lines(mixcount ? mixcount : 1, (uint64_t)K * mix_units, ea ? ea : 1));
    uint64_t stage = 0;
    if (K > 1) {
      while (true) {
        stage = std::max<uint64_t>(Ca * ri.Wc, mode == 2 ? (2 * Ca * ri.Wm + 3) / 4 : 2 * Ca * ri.Wm);
        if (Rk * Cb * esz + units * stage * esz <= st->ctx->smem_optin || (ri.Wc == 1 && ri.Wm == 1)) break;
        if (ri.Wc > 1) ri.Wc /= 2;
        if (ri.Wm > 1 && 2 * Ca * ri.Wm > Ca * ri.Wc) ri.Wm /= 2;
      }
    }
    const size_t head = (size_t)(Rk * Cb * esz + units * stage * esz);
    const size_t smem = with_meta ? ((head + 15) & ~(size_t)15) + meta : head;
    // the kernels' static shared memory (kResidentStaticSmem) comes on top
    if (smem + kResidentStaticSmem <= st->ctx->smem_optin) {
      rl = ResidentLaunch{};
      rl.ninst = 1;
      rl.cluster = K;
      rl.warps_per_cta = wpc;
      rl.stage_elems = (uint32_t)stage;
      rl.meta_smem = (uint32_t)with_meta;
      rl.group = mode;
      rl.smem_bytes = smem < 1024 ? 1024 : smem;
      return true;
    }
  }
  return false;
}

// Most consecutive column-pair passes one window of update units may take.
constexpr uint32_t kMixWindowPasses = 8;
// Replica clusters a lean launch may have (QPE_STRATEGY_LEAN_UNITS).
constexpr uint32_t kMaxReplicas = 8;

// The column-pair update-unit schedule of `pr` for cluster K, wpc warps per CTA
// and group stages of `stage` elements, built from the device's index pool on
// first use and kept with the program. False if no pass could be scheduled.
static bool ensure_mix_units(const qpe_program* pr, uint32_t K, uint32_t wpc, uint32_t stage) {
  if (pr->mix_wp_words && pr->mix_K == K && pr->mix_wpc == wpc && pr->mix_stage == stage)
    return pr->mix_scheduled > 0;
  const HostProgram& hp = pr->hp;
  cudaStream_t s = pr->ctx->stream;
  std::vector<uint32_t> pool(hp.pool_words);
  QPE_CK(cudaMemcpyAsync(pool.data(), pr->pool.p, pool.size() * 4, cudaMemcpyDeviceToHost, s));
  QPE_CK(cudaStreamSynchronize(s));
  MixUnits mu;
  build_mix_units(hp, pool.data(), K, wpc, stage, kMixWindowPasses, mu);
  pr->mix_words.release();
  pr->mix_slot.release();
  if (mu.scheduled) {
    pr->mix_words.alloc(mu.words.size() * 4);
    pr->mix_slot.alloc(mu.pass_slot.size() * 4);
    QPE_CK(cudaMemcpyAsync(pr->mix_words.p, mu.words.data(), mu.words.size() * 4, cudaMemcpyHostToDevice, s));
    QPE_CK(cudaMemcpyAsync(pr->mix_slot.p, mu.pass_slot.data(), mu.pass_slot.size() * 4, cudaMemcpyHostToDevice, s));
    QPE_CK(cudaStreamSynchronize(s));
  }
  pr->mix_K = K;
  pr->mix_wpc = wpc;
  pr->mix_stage = stage;
  pr->mix_wp_words = mu.wp_words ? mu.wp_words : mix_wp_words(hp);
  pr->mix_scheduled = mu.scheduled;
  return mu.scheduled > 0;
}

// The per-line programs of the row and column passes of `pr` for this geometry
// and number of replicas, built on first use from the device's index pool and
// line strings and kept with the program. False if no pass has programs.
static bool ensure_line_units(const qpe_program* pr, uint32_t K, uint32_t wpc, uint32_t stage, uint32_t Rk,
                              uint32_t replicas) {
  const uint32_t key[5] = {K, wpc, stage, Rk, replicas};
  if (std::equal(key, key + 5, pr->line_key)) return pr->line_passes > 0;
  const HostProgram& hp = pr->hp;
  cudaStream_t s = pr->ctx->stream;
  std::vector<uint32_t> pool(hp.pool_words), strA(hp.Ca), strB(hp.Cb);
  QPE_CK(cudaMemcpyAsync(pool.data(), pr->pool.p, pool.size() * 4, cudaMemcpyDeviceToHost, s));
  QPE_CK(cudaMemcpyAsync(strA.data(), pr->strA.p, strA.size() * 4, cudaMemcpyDeviceToHost, s));
  QPE_CK(cudaMemcpyAsync(strB.data(), pr->strB.p, strB.size() * 4, cudaMemcpyDeviceToHost, s));
  QPE_CK(cudaStreamSynchronize(s));
  LineUnits lu;
  build_line_units(hp, pool.data(), strA.data(), strB.data(), K, wpc, Rk, replicas, stage, lu);
  pr->line_words.release();
  pr->line_offs.release();
  pr->line_slot.release();
  if (lu.passes) {
    pr->line_words.alloc(lu.words.size() * 4);
    pr->line_offs.alloc(lu.offs.size() * 4);
    pr->line_slot.alloc(lu.pass_slot.size() * 4);
    QPE_CK(cudaMemcpyAsync(pr->line_words.p, lu.words.data(), lu.words.size() * 4, cudaMemcpyHostToDevice, s));
    QPE_CK(cudaMemcpyAsync(pr->line_offs.p, lu.offs.data(), lu.offs.size() * 4, cudaMemcpyHostToDevice, s));
    QPE_CK(cudaMemcpyAsync(pr->line_slot.p, lu.pass_slot.data(), lu.pass_slot.size() * 4, cudaMemcpyHostToDevice, s));
    QPE_CK(cudaStreamSynchronize(s));
  }
  std::copy(key, key + 5, pr->line_key);
  pr->line_passes = lu.passes;
  return lu.passes > 0;
}

static void run_resident(qpe_state* st, const qpe_program* pr, uint32_t K, uint32_t first, uint32_t last,
                         bool exact, bool in_place = false, uint32_t mode = 0, uint32_t replicas = 1) {
  ResidentLaunch rl;
  ResidentInstance ri{};
  if (!plan_resident(pr, st, K, rl, ri, mode))
    throw Error(QPE_ERR_UNSUPPORTED, "block does not fit the cluster's shared memory");
  if (replicas > 1) {
    // replica clusters of the lean kernel, each holding the whole block
    if (rl.group != 3 || K < 2) throw Error(QPE_ERR_INVALID, "replicas need a three-warp-group cluster of 2 or more");
    if (replicas > kMaxReplicas) throw Error(QPE_ERR_INVALID, "at most 8 replicas");
    if (st->xbuf.bytes < 2 * st->ld * st->esz) st->xbuf.alloc(2 * st->ld * st->esz);
    if (!st->xflag.p) st->xflag.alloc(16 * kMaxReplicas * sizeof(uint32_t));
    QPE_CK(cudaMemsetAsync(st->xflag.p, 0, st->xflag.bytes, st->ctx->stream));
    rl.replicas = replicas;
    ri.replicas = replicas;
    ri.xbuf = st->xbuf.p;
    ri.xflag = st->xflag.as<uint32_t>();
  }
  ri.err = st->ctx->err.as<int>();
  if (mode == 4 && ensure_mix_units(pr, K, rl.warps_per_cta, rl.stage_elems)) {
    ri.mix_words = pr->mix_words.as<uint32_t>();
    ri.mix_slot = pr->mix_slot.as<uint32_t>();
    ri.mix_wp_words = pr->mix_wp_words;
  }
  if (mode == 4 && K > 1 &&
      ensure_line_units(pr, K, rl.warps_per_cta, rl.stage_elems, ri.rows_per_cta, std::max(replicas, 1u))) {
    ri.line_slot = pr->line_slot.as<uint32_t>();
    ri.line_offs = pr->line_offs.as<uint32_t>();
    ri.line_words = pr->line_words.as<uint32_t>();
  }
  ri.state = st->data.p;
  ri.pool = pr->pool.as<uint32_t>();
  ri.ops = pr->ops.as<DevOp>();
  ri.coef = pr->coef.as<double>();
  ri.passes = pr->passes.as<Pass>();
  ri.strA = pr->strA.as<uint32_t>();
  ri.strB = pr->strB.as<uint32_t>();
  ri.npasses = (uint32_t)pr->hp.passes.size();
  ri.nops = (uint32_t)pr->hp.ops.size();
  ri.pool_words = (uint32_t)pr->hp.pool_words;
  ri.first = first;
  ri.last = last;
  ri.steps = pr->hp.steps;
  ri.order = pr->hp.order;
  ri.in_place = in_place ? 1u : 0u;
  if (!st->res_inst.p) st->res_inst.alloc(sizeof(ResidentInstance));
  QPE_CK(cudaMemcpyAsync(st->res_inst.p, &ri, sizeof(ri), cudaMemcpyHostToDevice, st->ctx->stream));
  rl.insts = st->res_inst.as<ResidentInstance>();
  // Leave the rest of the unified L1 / shared memory to L1, which then holds the
  // program's terms and index tables across passes.
  const int pct = (int)std::min<size_t>(100, (rl.smem_bytes * 100 + st->ctx->smem_optin - 1) / st->ctx->smem_optin + 1);
  QPE_CK(set_resident_carveout(st->dtype, exact, pct));
  QPE_CK(launch_resident(rl, st->dtype, exact, st->ctx->stream));
}

static void evolve_tiled(qpe_state* st, const qpe_program* pr, uint32_t first, uint32_t last, bool exact,
                         bool in_place = false);

// ResidentLaunch::group of a resident strategy.
static uint32_t resident_mode(uint32_t strategy) {
  if (strategy == QPE_STRATEGY_GROUP) return 1u;
  if (strategy == QPE_STRATEGY_HYBRID) return 2u;
  if (strategy == QPE_STRATEGY_LEAN) return 3u;
  if (strategy == QPE_STRATEGY_LEAN_UNITS) return 4u;
  return 0u;
}

// Strategy for (program, state): explicit, or timed on one power per candidate.
static void choose_strategy(qpe_state* st, const qpe_program* pr, const qpe_evolve_opts* opts, bool exact,
                            uint32_t& strategy, uint32_t& K, uint32_t& replicas) {
  strategy = opts ? opts->strategy : QPE_STRATEGY_AUTO;
  K = opts ? opts->cluster_size : 0;
  replicas = (opts && opts->replicas && strategy == QPE_STRATEGY_LEAN_UNITS) ? opts->replicas : 1u;
  ResidentLaunch rl;
  ResidentInstance ri{};
  if (strategy == QPE_STRATEGY_RESIDENT) {
    K = 1;
    return;
  }
  if (strategy == QPE_STRATEGY_CLUSTER || strategy == QPE_STRATEGY_GROUP || strategy == QPE_STRATEGY_HYBRID ||
      strategy == QPE_STRATEGY_LEAN || strategy == QPE_STRATEGY_LEAN_UNITS) {
    const uint32_t mode = resident_mode(strategy);
    if (K == 0) {
      for (uint32_t c = mode ? 1 : 2; c <= 16 && !K; c *= 2)
        if (plan_resident(pr, st, c, rl, ri, mode)) K = c;
      if (!K) throw Error(QPE_ERR_UNSUPPORTED, "block does not fit a cluster of 16");
    }
    return;
  }
  if (strategy == QPE_STRATEGY_TILED) return;
  if (st->tuned_prog == pr->id && st->tuned_exact == (uint32_t)exact) {
    strategy = st->tuned_strategy;
    K = st->tuned_cluster;
    replicas = st->tuned_replicas;
    return;
  }
  // Autotune: time one power of every feasible candidate, the tiled strategy
  // included. The trial powers write block 1, which is saved first and put back
  // afterwards, so that tuning leaves the register as it was.
  DevBuf saved;
  saved.alloc(st->ld * st->esz);
  char* block1 = st->data.as<char>() + st->ld * st->esz;
  QPE_CK(cudaMemcpyAsync(saved.p, block1, st->ld * st->esz, cudaMemcpyDeviceToDevice, st->ctx->stream));
  struct Restore {
    void* dst; const void* src; size_t n; cudaStream_t s;
    ~Restore() { cudaMemcpyAsync(dst, src, n, cudaMemcpyDeviceToDevice, s); cudaStreamSynchronize(s); }
  } restore{block1, saved.p, st->ld * st->esz, st->ctx->stream};
  struct Cand {
    uint32_t strategy, K, replicas;
  };
  std::vector<Cand> cands;
  for (uint32_t c = 1; c <= 16; c *= 2) {
    const uint32_t one = 1;
    if (plan_resident(pr, st, c, rl, ri))
      cands.push_back({c == 1 ? (uint32_t)QPE_STRATEGY_RESIDENT : (uint32_t)QPE_STRATEGY_CLUSTER, c, one});
    if (plan_resident(pr, st, c, rl, ri, 1)) cands.push_back({(uint32_t)QPE_STRATEGY_GROUP, c, one});
    if (plan_resident(pr, st, c, rl, ri, 2)) cands.push_back({(uint32_t)QPE_STRATEGY_HYBRID, c, one});
    if (plan_resident(pr, st, c, rl, ri, 3)) cands.push_back({(uint32_t)QPE_STRATEGY_LEAN, c, one});
    if (plan_resident(pr, st, c, rl, ri, 4) && ensure_mix_units(pr, c, rl.warps_per_cta, rl.stage_elems))
      for (uint32_t r = 1; r <= (c >= 8 ? 5u : 1u); ++r) cands.push_back({(uint32_t)QPE_STRATEGY_LEAN_UNITS, c, r});
  }
  cands.push_back({(uint32_t)QPE_STRATEGY_TILED, 0u, 1u});
  if (cands.size() == 1) {
    strategy = QPE_STRATEGY_TILED;
  } else {
    cudaEvent_t e0, e1;
    QPE_CK(cudaEventCreate(&e0));
    QPE_CK(cudaEventCreate(&e1));
    float best = 1e30f;
    for (auto& c : cands) {
      float ms = 0;
      auto run = [&]() {
        if (c.strategy == QPE_STRATEGY_TILED) evolve_tiled(st, pr, 1, 2, exact);
        else run_resident(st, pr, c.K, 1, 2, exact, false, resident_mode(c.strategy), c.replicas);
        if (c.replicas > 1) check_device_error(st->ctx);
      };
      try {
        run();  // warm-up of this configuration
        QPE_CK(cudaEventRecord(e0, st->ctx->stream));
        run();
        QPE_CK(cudaEventRecord(e1, st->ctx->stream));
        QPE_CK(cudaEventSynchronize(e1));
        QPE_CK(cudaEventElapsedTime(&ms, e0, e1));
      } catch (const Error&) {
        // A configuration the device cannot launch (e.g. too many CTAs per
        // cluster for the resources) is skipped; a sticky fault is not.
        if (cudaPeekAtLastError() != cudaSuccess) cudaGetLastError();
        if (cudaStreamQuery(st->ctx->stream) != cudaSuccess && cudaStreamQuery(st->ctx->stream) != cudaErrorNotReady) throw;
        continue;
      }
      if (ms < best) {
        best = ms;
        strategy = c.strategy;
        K = c.K;
        replicas = c.replicas;
      }
    }
    if (best == 1e30f) strategy = QPE_STRATEGY_TILED;
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
  }
  st->tuned_prog = pr->id;
  st->tuned_exact = exact;
  st->tuned_strategy = strategy;
  st->tuned_cluster = K;
  st->tuned_replicas = replicas;
}

static void evolve(qpe_state* st, const qpe_program* pr, const qpe_evolve_opts* opts) {
  const HostProgram& hp = pr->hp;
  if (hp.M != st->M || hp.na != st->na || hp.nb != st->nb)
    throw Error(QPE_ERR_INVALID, "program and state shapes differ");
  const bool in_place = opts && (opts->flags & QPE_EVOLVE_IN_PLACE);
  uint32_t first = 1, last = (uint32_t)st->N;
  if (in_place) {
    // Block first_power, evolved `repeats` times: the kernels see the range
    // [first, first + repeats) and write every power back to block first.
    first = opts->first_power;
    const uint32_t reps = opts->repeats ? opts->repeats : 1u;
    if (first >= st->N) throw Error(QPE_ERR_INVALID, "in-place block outside 0 .. 2^P - 1");
    if (reps > (1u << 30)) throw Error(QPE_ERR_INVALID, "repeats above 2^30");
    last = first + reps;
  } else {
    if (opts && (opts->first_power || opts->last_power)) {
      first = opts->first_power;
      last = opts->last_power;
    }
    if (first < 1 || last > st->N || first > last) throw Error(QPE_ERR_INVALID, "power range outside 1 .. 2^P");
  }
  st->probs_valid = false;
  if (first == last) return;
  const bool exact = st->dtype == QPE_C128 && !(opts && (opts->flags & QPE_EVOLVE_FP64_CONTRACT));
  uint32_t strategy = 0, K = 0, replicas = 1;
  choose_strategy(st, pr, opts, exact, strategy, K, replicas);
  st->last_strategy = strategy;
  st->last_cluster = strategy == QPE_STRATEGY_TILED ? 0 : K;
  st->last_replicas = replicas;
  if (strategy == QPE_STRATEGY_TILED) {
    evolve_tiled(st, pr, first, last, exact, in_place);
  } else {
    run_resident(st, pr, K, first, last, exact, in_place, resident_mode(strategy), replicas);
    QPE_CK(cudaStreamSynchronize(st->ctx->stream));
    if (replicas > 1) check_device_error(st->ctx);
  }
}

// Global-memory working block, one kernel launch per pass, one captured graph
// per controlled power replayed for every power.
static void evolve_tiled(qpe_state* st, const qpe_program* pr, uint32_t first, uint32_t last, bool exact,
                         bool in_place) {
  const HostProgram& hp = pr->hp;
  cudaStream_t s = st->ctx->stream;
  if (!st->work.p) st->work.alloc(st->ld * st->esz);
  // Working block (stored by columns) <- block first - 1 (block first when
  // evolving in place).
  const uint32_t src = in_place ? first : first - 1;
  QPE_CK(launch_load(st->work.p, st->data.p, (uint32_t)hp.Ca, (uint32_t)hp.Cb, src, st->dtype, s));
  k_set_int<<<1, 1, 0, s>>>(st->dk.as<int>(), (int)first);
  QPE_CK(cudaGetLastError());
  if (st->graph_prog != pr->id || st->graph_exact != (uint32_t)exact || !st->graph) {
    if (st->graph) cudaGraphExecDestroy(st->graph);
    st->graph = nullptr;
    st->graph_prog = 0;
    std::vector<PassLaunch> plans;
    size_t max_smem = 0;
    for (uint32_t sw = 0; sw < hp.steps * hp.order; ++sw) {
      const bool rev = hp.order == 2 && (sw & 1);
      for (size_t pj = 0; pj < hp.passes.size(); ++pj) {
        const Pass& pass = hp.passes[rev ? hp.passes.size() - 1 - pj : pj];
        plans.push_back(plan_pass(pr, st, pass));
        PassLaunch& pl = plans.back();
        pl.rev = rev ? 1u : 0u;
        pl.exact = exact ? 1u : 0u;
        const size_t sm = pass_smem_bytes(pl, st->esz);
        if (sm > max_smem) max_smem = sm;
      }
    }
    QPE_CK(configure_pass_kernels(st->dtype, max_smem < 48 * 1024 ? 48 * 1024 : max_smem));
    cudaGraph_t g = nullptr;
    QPE_CK(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
    cudaError_t cap_err = cudaSuccess;
    for (const PassLaunch& pl : plans)
      if (cap_err == cudaSuccess) cap_err = launch_pass(pl, st->dtype, s);
    if (cap_err == cudaSuccess)
      cap_err = launch_snapshot(st->work.p, st->data.p, (uint32_t)hp.Ca, (uint32_t)hp.Cb, st->dk.as<int>(), st->dtype, s);
    if (cap_err == cudaSuccess) cap_err = launch_advance(st->dk.as<int>(), s);
    cudaError_t end_err = cudaStreamEndCapture(s, &g);
    if (cap_err != cudaSuccess) {
      if (g) cudaGraphDestroy(g);
      QPE_CK(cap_err);
    }
    QPE_CK(end_err);
    cudaGraphExec_t ge = nullptr;
    cudaError_t ie = cudaGraphInstantiate(&ge, g, 0);
    cudaGraphDestroy(g);
    QPE_CK(ie);
    st->graph = ge;
    st->graph_prog = pr->id;
    st->graph_exact = exact;
  }
  for (uint32_t k = first; k < last; ++k) {
    // In place, every power's snapshot targets block first again.
    if (in_place && k > first) {
      k_set_int<<<1, 1, 0, s>>>(st->dk.as<int>(), (int)first);
      QPE_CK(cudaGetLastError());
    }
    QPE_CK(cudaGraphLaunch(st->graph, s));
  }
  QPE_CK(cudaStreamSynchronize(s));
}

static void qift(qpe_state* st) {
  cudaStream_t s = st->ctx->stream;
  const double norm = std::sqrt((double)st->N);
  QPE_CK(launch_qift(st->data.p, st->ld, st->P, st->tw.p, norm, st->partial.as<double>(), st->qift_grid, st->qift_T,
                     st->dtype, s));
  QPE_CK(launch_reduce_partials(st->partial.as<double>(), st->qift_grid, (uint32_t)st->N, st->probs.as<double>(), s));
  QPE_CK(cudaStreamSynchronize(s));
  st->probs_valid = true;
}

static void check_state(qpe_state* st) {
  if (!st) throw Error(QPE_ERR_INVALID, "null state");
  use_device(st->ctx);
}

static TermArrays term_arrays(const qpe_term* pp, size_t n_pp, const qpe_term* pq, size_t n_pq,
                              const qpe_term* pqqp, size_t n_pqqp, const qpe_term* pqqr, size_t n_pqqr,
                              const qpe_term* pqrs, size_t n_pqrs) {
  TermArrays T{{pp, pq, pqqp, pqqr, pqrs}, {n_pp, n_pq, n_pqqp, n_pqqr, n_pqrs}};
  for (int i = 0; i < 5; ++i)
    if (T.n[i] && !T.t[i]) throw Error(QPE_ERR_INVALID, "null term array with nonzero count");
  return T;
}

}  // namespace qpe

extern "C" {

int qpe_version(void) { return 1; }

const char* qpe_last_error(void) { return qpe::g_last_error.c_str(); }

int qpe_device_count(int* count) {
  return guard([&] {
    if (!count) throw Error(QPE_ERR_INVALID, "null argument");
    int n = 0;
    cudaError_t e = cudaGetDeviceCount(&n);
    if (e != cudaSuccess) {
      cudaGetLastError();
      n = 0;
    }
    *count = n;
  });
}

int qpe_context_create(int device, qpe_context** out) {
  return guard([&] {
    if (!out) throw Error(QPE_ERR_INVALID, "null output pointer");
    *out = nullptr;
    int n = 0;
    cudaError_t e = cudaGetDeviceCount(&n);
    if (e != cudaSuccess || n == 0) {
      cudaGetLastError();
      throw Error(QPE_ERR_NO_DEVICE, "no CUDA device available");
    }
    if (device < 0 || device >= n) throw Error(QPE_ERR_INVALID, "device index out of range");
    auto ctx = new qpe_context();
    try {
      ctx->device = device;
      QPE_CK(cudaSetDevice(device));
      cudaDeviceProp prop;
      QPE_CK(cudaGetDeviceProperties(&prop, device));
      if (prop.major < 10) throw Error(QPE_ERR_UNSUPPORTED, "this library is built for sm_103a (GB300)");
      ctx->num_sms = prop.multiProcessorCount;
      ctx->smem_optin = prop.sharedMemPerBlockOptin;
      QPE_CK(cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking));
      std::vector<uint64_t> tb(64 * BINOM_K);
      host_ref_binom_table(tb.data());
      ctx->binom.alloc(tb.size() * sizeof(uint64_t));
      QPE_CK(cudaMemcpy(ctx->binom.p, tb.data(), tb.size() * sizeof(uint64_t), cudaMemcpyHostToDevice));
      ctx->err.alloc(16);
      QPE_CK(cudaMemset(ctx->err.p, 0, 16));
    } catch (...) {
      if (ctx->stream) cudaStreamDestroy(ctx->stream);
      delete ctx;
      throw;
    }
    *out = ctx;
  });
}

int qpe_context_destroy(qpe_context* ctx) {
  if (!ctx) return QPE_OK;
  cudaSetDevice(ctx->device);
  for (cudaEvent_t& e : ctx->events)
    if (e) cudaEventDestroy(e);
  if (ctx->stream) {
    cudaStreamSynchronize(ctx->stream);
    cudaStreamDestroy(ctx->stream);
  }
  delete ctx;
  return QPE_OK;
}

int qpe_synchronize(qpe_context* ctx) {
  return guard([&] {
    check_ctx(ctx);
    QPE_CK(cudaStreamSynchronize(ctx->stream));
    check_device_error(ctx);
  });
}

int qpe_timer_record(qpe_context* ctx, uint32_t slot) {
  return guard([&] {
    check_ctx(ctx);
    if (slot >= 16) throw Error(QPE_ERR_INVALID, "timer slot must be < 16");
    if (!ctx->events[slot]) QPE_CK(cudaEventCreate(&ctx->events[slot]));
    QPE_CK(cudaEventRecord(ctx->events[slot], ctx->stream));
  });
}

int qpe_timer_elapsed_ms(qpe_context* ctx, uint32_t a, uint32_t b, float* ms) {
  return guard([&] {
    check_ctx(ctx);
    if (a >= 16 || b >= 16 || !ctx->events[a] || !ctx->events[b] || !ms)
      throw Error(QPE_ERR_INVALID, "timer slots not recorded");
    QPE_CK(cudaEventSynchronize(ctx->events[b]));
    QPE_CK(cudaEventElapsedTime(ms, ctx->events[a], ctx->events[b]));
  });
}

int qpe_flush_l2(qpe_context* ctx) {
  return guard([&] {
    check_ctx(ctx);
    if (!ctx->flush.p) ctx->flush.alloc(256ull << 20);
    QPE_CK(cudaMemsetAsync(ctx->flush.p, 0x5a, ctx->flush.bytes, ctx->stream));
  });
}

int qpe_measure_fp64_peak(qpe_context* ctx, double* tflops) {
  return guard([&] {
    check_ctx(ctx);
    if (!tflops) throw Error(QPE_ERR_INVALID, "null output");
    DevBuf out;
    const uint32_t ctas = (uint32_t)ctx->num_sms * 4, threads = 256, iters = 4096;
    out.alloc((size_t)ctas * threads * sizeof(double));
    cudaEvent_t ev[2] = {};
    QPE_CK(cudaEventCreate(&ev[0]));
    struct Events {
      cudaEvent_t* e;
      ~Events() {
        for (int i = 0; i < 2; ++i)
          if (e[i]) cudaEventDestroy(e[i]);
      }
    } guard_events{ev};
    QPE_CK(cudaEventCreate(&ev[1]));
    QPE_CK(launch_fp64_fma_probe(out.as<double>(), ctas, threads, iters, ctx->stream));  // warm-up
    QPE_CK(cudaEventRecord(ev[0], ctx->stream));
    const int reps = 4;
    for (int r = 0; r < reps; ++r) QPE_CK(launch_fp64_fma_probe(out.as<double>(), ctas, threads, iters, ctx->stream));
    QPE_CK(cudaEventRecord(ev[1], ctx->stream));
    QPE_CK(cudaEventSynchronize(ev[1]));
    float ms = 0.f;
    QPE_CK(cudaEventElapsedTime(&ms, ev[0], ev[1]));
    const double flops = 2.0 * kFp64ProbeChains * (double)iters * ctas * threads * reps;
    *tflops = flops / (ms * 1e-3) / 1e12;
  });
}

int qpe_host_alloc(size_t bytes, void** out) {
  return guard([&] {
    if (!out) throw Error(QPE_ERR_INVALID, "null output");
    *out = nullptr;
    QPE_CK(cudaMallocHost(out, bytes ? bytes : 16));
  });
}

int qpe_host_free(void* p) {
  return guard([&] {
    if (p) QPE_CK(cudaFreeHost(p));
  });
}

int qpe_rank(qpe_context* ctx, const uint64_t* bvs, int64_t* ranks, size_t n) {
  return guard([&] {
    check_ctx(ctx);
    if (n && (!bvs || !ranks)) throw Error(QPE_ERR_INVALID, "null argument");
    if (!n) return;
    DevBuf a, b;
    a.alloc(n * 8);
    b.alloc(n * 8);
    QPE_CK(cudaMemcpyAsync(a.p, bvs, n * 8, cudaMemcpyHostToDevice, ctx->stream));
    QPE_CK(launch_rank(ctx->binom.as<uint64_t>(), a.as<uint64_t>(), b.as<int64_t>(), n, ctx->stream));
    QPE_CK(cudaMemcpyAsync(ranks, b.p, n * 8, cudaMemcpyDeviceToHost, ctx->stream));
    QPE_CK(cudaStreamSynchronize(ctx->stream));
  });
}

int qpe_unrank(qpe_context* ctx, uint32_t nbits, uint32_t weight, const int64_t* ranks, uint64_t* bvs, size_t n) {
  return guard([&] {
    check_ctx(ctx);
    if (n && (!bvs || !ranks)) throw Error(QPE_ERR_INVALID, "null argument");
    if (nbits == 0 || nbits > 32 || weight > nbits) throw Error(QPE_ERR_INVALID, "need 0 < nbits <= 32, weight <= nbits");
    const uint64_t total = binom((int)nbits, (int)weight);
    for (size_t i = 0; i < n; ++i)
      if (ranks[i] < 0 || (uint64_t)ranks[i] >= total) throw Error(QPE_ERR_INVALID, "rank out of range");
    if (!n) return;
    DevBuf a, b;
    a.alloc(n * 8);
    b.alloc(n * 8);
    QPE_CK(cudaMemcpyAsync(a.p, ranks, n * 8, cudaMemcpyHostToDevice, ctx->stream));
    QPE_CK(launch_unrank(ctx->binom.as<uint64_t>(), nbits, weight, a.as<int64_t>(), b.as<uint64_t>(), n, ctx->stream));
    QPE_CK(cudaMemcpyAsync(bvs, b.p, n * 8, cudaMemcpyDeviceToHost, ctx->stream));
    QPE_CK(cudaStreamSynchronize(ctx->stream));
  });
}

int qpe_rank_with_swaps(qpe_context* ctx, uint32_t nbits, uint64_t bv, const uint32_t* swaps, int64_t* ranks,
                        size_t nq) {
  return guard([&] {
    check_ctx(ctx);
    if (nq && (!swaps || !ranks)) throw Error(QPE_ERR_INVALID, "null argument");
    if (nbits == 0 || nbits > 63) throw Error(QPE_ERR_INVALID, "need 0 < nbits <= 63");
    if (nbits < 64 && (bv >> nbits) != 0) throw Error(QPE_ERR_INVALID, "bit vector wider than nbits");
    for (size_t i = 0; i < nq; ++i) {
      const uint32_t* q = swaps + 4 * i;
      if (q[0] >= nbits || q[1] >= nbits || (q[2] != 0xffffffffu && (q[2] >= nbits || q[3] >= nbits)))
        throw Error(QPE_ERR_INVALID, "swap position out of range");
    }
    if (!nq) return;
    DevBuf a, b;
    a.alloc(nq * 16);
    b.alloc(nq * 8);
    QPE_CK(cudaMemcpyAsync(a.p, swaps, nq * 16, cudaMemcpyHostToDevice, ctx->stream));
    QPE_CK(launch_rank_with_swaps(ctx->binom.as<uint64_t>(), nbits, bv, a.as<uint32_t>(), b.as<int64_t>(), nq,
                                  ctx->stream));
    QPE_CK(cudaMemcpyAsync(ranks, b.p, nq * 8, cudaMemcpyDeviceToHost, ctx->stream));
    QPE_CK(cudaStreamSynchronize(ctx->stream));
  });
}

int qpe_axis_table(qpe_context* ctx, int kind, uint32_t nbits, uint32_t weight, const uint32_t* orbitals,
                   uint32_t* i01, uint32_t* i10, uint8_t* parity, size_t cap, size_t* count) {
  return guard([&] {
    check_ctx(ctx);
    if (!orbitals || !count) throw Error(QPE_ERR_INVALID, "null argument");
    if (kind < 0 || kind > 4) throw Error(QPE_ERR_INVALID, "unknown table kind");
    if (nbits == 0 || nbits > 31 || weight > nbits) throw Error(QPE_ERR_INVALID, "need 0 < nbits <= 31, weight <= nbits");
    static const int nfix[5] = {1, 2, 2, 3, 4}, nocc[5] = {1, 2, 1, 2, 2};
    AxisTable t{};
    t.kind = (uint8_t)kind;
    t.nbits = (uint8_t)nbits;
    t.weight = (uint8_t)weight;
    t.nfixed = (uint8_t)nfix[kind];
    for (int i = 0; i < nfix[kind]; ++i) {
      if (orbitals[i] >= nbits) throw Error(QPE_ERR_INVALID, "orbital out of range");
      for (int j = 0; j < i; ++j)
        if (orbitals[j] == orbitals[i]) throw Error(QPE_ERR_INVALID, "orbitals repeat");
      t.o[i] = (uint8_t)orbitals[i];
    }
    const uint64_t n = binom((int)nbits - nfix[kind], (int)weight - nocc[kind]);
    *count = (size_t)n;
    if (n > cap) throw Error(QPE_ERR_INVALID, "output capacity too small");
    if (n == 0) return;
    if (n > 0x7fffffffull) throw Error(QPE_ERR_UNSUPPORTED, "table too large");
    if (!i01 || ((kind == 2 || kind == 3 || kind == 4) && (!i10 || !parity))) throw Error(QPE_ERR_INVALID, "null output");
    t.count = (uint32_t)n;
    const bool pairs = kind >= 2;
    DevBuf tabs, start, pool;
    tabs.alloc(sizeof(AxisTable));
    start.alloc(2 * sizeof(uint32_t));
    pool.alloc(n * (pairs ? 8 : 4));
    uint32_t st[2] = {0, (uint32_t)n};
    QPE_CK(cudaMemcpyAsync(tabs.p, &t, sizeof(t), cudaMemcpyHostToDevice, ctx->stream));
    QPE_CK(cudaMemcpyAsync(start.p, st, sizeof(st), cudaMemcpyHostToDevice, ctx->stream));
    QPE_CK(launch_build_tables(ctx->binom.as<uint64_t>(), tabs.as<AxisTable>(), start.as<uint32_t>(), 1, n,
                               pool.as<uint32_t>(), ctx->stream));
    std::vector<uint32_t> h(n * (pairs ? 2 : 1));
    QPE_CK(cudaMemcpyAsync(h.data(), pool.p, h.size() * 4, cudaMemcpyDeviceToHost, ctx->stream));
    QPE_CK(cudaStreamSynchronize(ctx->stream));
    for (uint64_t j = 0; j < n; ++j) {
      if (pairs) {
        i01[j] = h[2 * j] & 0x7fffffffu;
        parity[j] = (uint8_t)(h[2 * j] >> 31);
        i10[j] = h[2 * j + 1];
      } else {
        i01[j] = h[j];
        if (parity) parity[j] = 0;
      }
    }
  });
}

int qpe_program_create(qpe_context* ctx, uint32_t M, uint32_t na, uint32_t nb, const qpe_term* pp, size_t n_pp,
                       const qpe_term* pq, size_t n_pq, const qpe_term* pqqp, size_t n_pqqp, const qpe_term* pqqr,
                       size_t n_pqqr, const qpe_term* pqrs, size_t n_pqrs, uint32_t order, uint32_t steps,
                       qpe_program** out) {
  return guard([&] {
    check_ctx(ctx);
    if (!out) throw Error(QPE_ERR_INVALID, "null output pointer");
    *out = nullptr;
    TermArrays T = term_arrays(pp, n_pp, pq, n_pq, pqqp, n_pqqp, pqqr, n_pqqr, pqrs, n_pqrs);
    auto pr = new qpe_program();
    try {
      static std::atomic<uint64_t> next_id{1};
      pr->ctx = ctx;
      pr->id = next_id++;
      build_program(pr->hp, M, na, nb, T, order, steps);
      build_device_program(pr);
    } catch (...) {
      delete pr;
      throw;
    }
    *out = pr;
  });
}

int qpe_program_destroy(qpe_program* pr) {
  if (!pr) return QPE_OK;
  cudaSetDevice(pr->ctx->device);
  delete pr;
  return QPE_OK;
}

static void fill_info(const HostProgram& hp, qpe_program_info* info);

int qpe_program_plan(uint32_t M, uint32_t na, uint32_t nb, const qpe_term* pp, size_t n_pp, const qpe_term* pq,
                     size_t n_pq, const qpe_term* pqqp, size_t n_pqqp, const qpe_term* pqqr, size_t n_pqqr,
                     const qpe_term* pqrs, size_t n_pqrs, uint32_t order, uint32_t steps, qpe_program_info* info) {
  return guard([&] {
    if (!info) throw Error(QPE_ERR_INVALID, "null output");
    TermArrays T = term_arrays(pp, n_pp, pq, n_pq, pqqp, n_pqqp, pqqr, n_pqqr, pqrs, n_pqrs);
    HostProgram hp;
    build_program(hp, M, na, nb, T, order, steps);
    fill_info(hp, info);
  });
}

int qpe_program_get_info(const qpe_program* pr, qpe_program_info* info) {
  if (!pr || !info) return fail(QPE_ERR_INVALID, "null argument");
  fill_info(pr->hp, info);
  return QPE_OK;
}

int qpe_program_unit_schedule(const qpe_program* pr, uint32_t* cluster_size, uint32_t* scheduled_passes) {
  if (!pr || !cluster_size || !scheduled_passes) return fail(QPE_ERR_INVALID, "null argument");
  *cluster_size = pr->mix_wp_words ? pr->mix_K : 0u;
  *scheduled_passes = pr->mix_wp_words ? pr->mix_scheduled : 0u;
  return QPE_OK;
}

static void fill_info(const HostProgram& hp, qpe_program_info* info) {
  info->num_orbitals = hp.M;
  info->n_alpha = hp.na;
  info->n_beta = hp.nb;
  info->c_alpha = (uint32_t)hp.Ca;
  info->c_beta = (uint32_t)hp.Cb;
  info->num_ops = hp.ops_per_sweep;
  info->num_ops_per_power = (uint32_t)(hp.ops.size() * hp.steps * hp.order);
  info->touches_per_sweep = hp.touches_per_sweep;
  info->touches_per_power = hp.touches_per_power;
  uint64_t entries = 0;
  for (const AxisTable& t : hp.tables) entries += t.count;
  info->table_entries = entries;
  info->num_passes_per_power = (uint32_t)(hp.passes.size() * hp.steps * hp.order);
  info->reserved = 0;
}

int qpe_state_create(qpe_context* ctx, uint32_t M, uint32_t na, uint32_t nb, uint32_t P, int dtype, qpe_state** out) {
  return guard([&] {
    check_ctx(ctx);
    if (!out) throw Error(QPE_ERR_INVALID, "null output pointer");
    *out = nullptr;
    if (M == 0 || M > 31 || na == 0 || nb == 0 || na > M || nb > M) throw Error(QPE_ERR_INVALID, "bad shape");
    if (P == 0 || P > 13) throw Error(QPE_ERR_UNSUPPORTED, "precision must be in 1..13");
    if (dtype != QPE_C128 && dtype != QPE_C64) throw Error(QPE_ERR_INVALID, "unknown dtype");
    auto st = new qpe_state();
    try {
      st->ctx = ctx;
      st->M = M;
      st->na = na;
      st->nb = nb;
      st->P = P;
      st->dtype = dtype;
      st->Ca = binom((int)M, (int)na);
      st->Cb = binom((int)M, (int)nb);
      st->ld = st->Ca * st->Cb;
      state_alloc(st);
      QPE_CK(cudaMemsetAsync(st->data.p, 0, st->data.bytes, ctx->stream));
      QPE_CK(cudaStreamSynchronize(ctx->stream));
    } catch (...) {
      delete st;
      throw;
    }
    *out = st;
  });
}

int qpe_state_destroy(qpe_state* st) {
  if (!st) return QPE_OK;
  cudaSetDevice(st->ctx->device);
  delete st;
  return QPE_OK;
}

int qpe_state_upload(qpe_state* st, const void* host, uint64_t first, uint64_t count) {
  return guard([&] {
    check_state(st);
    if (count && !host) throw Error(QPE_ERR_INVALID, "null host pointer");
    if (first > st->N * st->ld || count > st->N * st->ld - first) throw Error(QPE_ERR_INVALID, "range outside the state");
    if (!count) return;
    QPE_CK(cudaMemcpyAsync(st->data.as<char>() + first * st->esz, host, count * st->esz, cudaMemcpyHostToDevice,
                           st->ctx->stream));
    QPE_CK(cudaStreamSynchronize(st->ctx->stream));
    st->probs_valid = false;
  });
}

int qpe_state_download(qpe_state* st, void* host, uint64_t first, uint64_t count) {
  return guard([&] {
    check_state(st);
    if (count && !host) throw Error(QPE_ERR_INVALID, "null host pointer");
    if (first > st->N * st->ld || count > st->N * st->ld - first) throw Error(QPE_ERR_INVALID, "range outside the state");
    if (!count) return;
    QPE_CK(cudaMemcpyAsync(host, st->data.as<char>() + first * st->esz, count * st->esz, cudaMemcpyDeviceToHost,
                           st->ctx->stream));
    QPE_CK(cudaStreamSynchronize(st->ctx->stream));
    check_device_error(st->ctx);
  });
}

int qpe_state_zero(qpe_state* st) {
  return guard([&] {
    check_state(st);
    QPE_CK(cudaMemsetAsync(st->data.p, 0, st->data.bytes, st->ctx->stream));
    QPE_CK(cudaStreamSynchronize(st->ctx->stream));
    st->probs_valid = false;
  });
}

int qpe_evolve(qpe_state* st, const qpe_program* pr, const qpe_evolve_opts* opts) {
  return guard([&] {
    check_state(st);
    if (!pr) throw Error(QPE_ERR_INVALID, "null program");
    if (opts && opts->strategy > QPE_STRATEGY_LEAN_UNITS) throw Error(QPE_ERR_INVALID, "unknown strategy");
    if (opts && opts->cluster_size && (opts->cluster_size > 16 || (opts->cluster_size & (opts->cluster_size - 1))))
      throw Error(QPE_ERR_INVALID, "cluster_size must be a power of two <= 16");
    if (opts && opts->replicas > 1 && opts->strategy != QPE_STRATEGY_LEAN_UNITS)
      throw Error(QPE_ERR_INVALID, "replicas need QPE_STRATEGY_LEAN_UNITS");
    if (opts && (opts->flags & ~(QPE_EVOLVE_FP64_CONTRACT | QPE_EVOLVE_IN_PLACE)))
      throw Error(QPE_ERR_INVALID, "unknown evolve flag");
    evolve(st, pr, opts);
  });
}

int qpe_state_qift(qpe_state* st) {
  return guard([&] {
    check_state(st);
    qift(st);
  });
}

int qpe_state_phase_probs(qpe_state* st, double* probs) {
  return guard([&] {
    check_state(st);
    if (!probs) throw Error(QPE_ERR_INVALID, "null output");
    if (!st->probs_valid) {
      QPE_CK(launch_block_sums(st->data.p, st->ld, (uint32_t)st->N, st->probs.as<double>(), st->dtype, st->ctx->stream));
    }
    QPE_CK(cudaMemcpyAsync(probs, st->probs.p, st->N * sizeof(double), cudaMemcpyDeviceToHost, st->ctx->stream));
    QPE_CK(cudaStreamSynchronize(st->ctx->stream));
    check_device_error(st->ctx);
  });
}

int qpe_state_last_replicas(const qpe_state* st, uint32_t* replicas) {
  if (!st || !replicas) return fail(QPE_ERR_INVALID, "null argument");
  *replicas = st->last_replicas;
  return QPE_OK;
}

int qpe_state_last_strategy(const qpe_state* st, uint32_t* strategy, uint32_t* cluster_size) {
  return guard([&] {
    if (!st || !strategy || !cluster_size) throw Error(QPE_ERR_INVALID, "null argument");
    *strategy = st->last_strategy;
    *cluster_size = st->last_cluster;
  });
}

int qpe_state_block_norms(qpe_state* st, double* norms) {
  return guard([&] {
    check_state(st);
    if (!norms) throw Error(QPE_ERR_INVALID, "null output");
    DevBuf tmp;
    tmp.alloc(st->N * sizeof(double));
    QPE_CK(launch_block_sums(st->data.p, st->ld, (uint32_t)st->N, tmp.as<double>(), st->dtype, st->ctx->stream));
    QPE_CK(cudaMemcpyAsync(norms, tmp.p, st->N * sizeof(double), cudaMemcpyDeviceToHost, st->ctx->stream));
    QPE_CK(cudaStreamSynchronize(st->ctx->stream));
  });
}

// ---- one-shot calls ----

int qpe_time_evolve_over_terms(qpe_context* ctx, uint32_t M, uint32_t e, uint32_t P, const qpe_term* pp, size_t n_pp,
                               const qpe_term* pq, size_t n_pq, const qpe_term* pqqp, size_t n_pqqp,
                               const qpe_term* pqqr, size_t n_pqqr, const qpe_term* pqrs, size_t n_pqrs,
                               double* state) {
  return guard([&] {
    check_ctx(ctx);
    if (!state) throw Error(QPE_ERR_INVALID, "null state");
    qpe_program* pr = nullptr;
    qpe_state* st = nullptr;
    int rc = qpe_program_create(ctx, M, e, e, pp, n_pp, pq, n_pq, pqqp, n_pqqp, pqqr, n_pqqr, pqrs, n_pqrs, 1, 1, &pr);
    if (rc) throw Error(rc, g_last_error);
    rc = qpe_state_create(ctx, M, e, e, P, QPE_C128, &st);
    if (rc) {
      qpe_program_destroy(pr);
      throw Error(rc, g_last_error);
    }
    const uint64_t ld = st->ld, total = st->N * ld;
    rc = qpe_state_upload(st, state, 0, ld);
    if (!rc) rc = qpe_evolve(st, pr, nullptr);
    if (!rc) rc = qpe_state_download(st, state, 0, total);
    std::string msg = g_last_error;
    qpe_state_destroy(st);
    qpe_program_destroy(pr);
    if (rc) throw Error(rc, msg);
  });
}

int qpe_time_evolve_iqpe(qpe_context* ctx, uint32_t M, uint32_t e, uint32_t P, const qpe_term* pp, size_t n_pp,
                         const qpe_term* pq, size_t n_pq, const qpe_term* pqqp, size_t n_pqqp, const qpe_term* pqqr,
                         size_t n_pqqr, const qpe_term* pqrs, size_t n_pqrs, uint32_t applications, double* state) {
  return guard([&] {
    check_ctx(ctx);
    if (!state) throw Error(QPE_ERR_INVALID, "null state");
    if (P == 0) throw Error(QPE_ERR_INVALID, "time_evolve_iqpe needs precision >= 1 (it evolves block 1)");
    if (applications == 0) return;
    qpe_program* pr = nullptr;
    qpe_state* st = nullptr;
    int rc = qpe_program_create(ctx, M, e, e, pp, n_pp, pq, n_pq, pqqp, n_pqqp, pqqr, n_pqqr, pqrs, n_pqrs,
                                1u | QPE_PROGRAM_APPLY_UNITARY_ORDER, 1, &pr);
    if (rc) throw Error(rc, g_last_error);
    // Only block 1 takes part: a two-block device register holds it.
    rc = qpe_state_create(ctx, M, e, e, 1, QPE_C128, &st);
    if (rc) {
      qpe_program_destroy(pr);
      throw Error(rc, g_last_error);
    }
    const uint64_t ld = st->ld;
    double* block1 = state + 2 * ld;
    rc = qpe_state_upload(st, block1, ld, ld);
    qpe_evolve_opts o{};
    o.flags = QPE_EVOLVE_IN_PLACE;
    o.first_power = 1;
    o.repeats = applications;
    if (!rc) rc = qpe_evolve(st, pr, &o);
    if (!rc) rc = qpe_state_download(st, block1, ld, ld);
    std::string msg = g_last_error;
    qpe_state_destroy(st);
    qpe_program_destroy(pr);
    if (rc) throw Error(rc, msg);
  });
}

static qpe_state* raw_state(qpe_context* ctx, uint32_t P, uint64_t ld) {
  if (P == 0 || P > 13) throw Error(QPE_ERR_UNSUPPORTED, "precision must be in 1..13");
  if (ld == 0) throw Error(QPE_ERR_INVALID, "ld must be positive");
  auto st = new qpe_state();
  try {
    st->ctx = ctx;
    st->P = P;
    st->dtype = QPE_C128;
    st->ld = ld;
    state_alloc(st);
  } catch (...) {
    delete st;
    throw;
  }
  return st;
}

int qpe_qift(qpe_context* ctx, uint32_t P, uint64_t ld, double* state) {
  return guard([&] {
    check_ctx(ctx);
    if (!state) throw Error(QPE_ERR_INVALID, "null state");
    qpe_state* st = raw_state(ctx, P, ld);
    try {
      const size_t bytes = st->N * ld * 16;
      QPE_CK(cudaMemcpyAsync(st->data.p, state, bytes, cudaMemcpyHostToDevice, ctx->stream));
      qift(st);
      QPE_CK(cudaMemcpyAsync(state, st->data.p, bytes, cudaMemcpyDeviceToHost, ctx->stream));
      QPE_CK(cudaStreamSynchronize(ctx->stream));
    } catch (...) {
      delete st;
      throw;
    }
    delete st;
  });
}

int qpe_identify_phase_amplitudes(qpe_context* ctx, uint32_t P, uint64_t ld, const double* state, double* probs) {
  return guard([&] {
    check_ctx(ctx);
    if (!state || !probs) throw Error(QPE_ERR_INVALID, "null argument");
    qpe_state* st = raw_state(ctx, P, ld);
    try {
      QPE_CK(cudaMemcpyAsync(st->data.p, state, st->N * ld * 16, cudaMemcpyHostToDevice, ctx->stream));
      QPE_CK(launch_block_sums(st->data.p, ld, (uint32_t)st->N, st->probs.as<double>(), QPE_C128, ctx->stream));
      QPE_CK(cudaMemcpyAsync(probs, st->probs.p, st->N * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
      QPE_CK(cudaStreamSynchronize(ctx->stream));
    } catch (...) {
      delete st;
      throw;
    }
    delete st;
  });
}

}  // extern "C"
