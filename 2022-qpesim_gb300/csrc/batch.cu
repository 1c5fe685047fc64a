// batch.cu - the batching form: many Hamiltonians evolved, transformed and read
// out by one launch of one CUDA graph.
//
// Instances whose programs have the same structure (same orbitals and electron
// counts, same terms, hence the same index tables, passes and term order, with
// every coefficient inline) form a class. A class keeps one copy of the tables
// and term list and one (c0, c1) coefficient pair per term per instance; each of
// its tile passes is a single launch over (instance, tile). The graph holds, per
// class and side by side, a conditional while-loop node whose body is one
// controlled power (the class's passes, the snapshot of every working block into
// its register, and a kernel that advances the power and sets the loop
// condition), followed by the QIFT and phase histogram of every instance. The
// tile shape of each class (lines per warp tile, warps per CTA) is picked by
// timing one power of every candidate.
#include <cuda_runtime.h>

#include <algorithm>
#include <deque>
#include <cmath>
#include <cstring>
#include <numeric>
#include <vector>

#include "abi_internal.h"

using namespace qpe;

namespace {

struct BatchClass {
  const qpe_program* shape = nullptr;  // tables, terms and passes shared by the class
  std::vector<uint32_t> members;       // instance indices, largest first
  uint64_t ld = 0;
  DevBuf icoef;                        // [member][term] (c0, c1)
  DevBuf works_ptr, states_ptr;        // device arrays of per-member pointers
  DevBuf dk;
  uint32_t W = 0, wpc = 4;             // tile shape (lines per column tile, 0 = default; warps per CTA)
  float tuned_ms = 0.f;                // one power of the class alone, best tile shape
  std::vector<PassLaunch> plans;       // one power: steps x sweeps of passes
};

bool same_structure(const HostProgram& a, const HostProgram& b) {
  if (a.M != b.M || a.na != b.na || a.nb != b.nb || a.order != b.order || a.steps != b.steps) return false;
  if (a.tables.size() != b.tables.size() || a.passes.size() != b.passes.size() || a.ops.size() != b.ops.size())
    return false;
  if (!a.tables.empty() && std::memcmp(a.tables.data(), b.tables.data(), a.tables.size() * sizeof(AxisTable)))
    return false;
  if (!a.passes.empty() && std::memcmp(a.passes.data(), b.passes.data(), a.passes.size() * sizeof(Pass))) return false;
  for (size_t i = 0; i < a.ops.size(); ++i) {
    const DevOp &x = a.ops[i], &y = b.ops[i];
    if (x.tab != y.tab || x.count != y.count || x.kind != y.kind || x.ncond != y.ncond || x.cb0 != y.cb0 ||
        x.cb1 != y.cb1 || x.gen != OP_INLINE || y.gen != OP_INLINE)
      return false;
  }
  return true;
}

}  // namespace

struct qpe_batch {
  qpe_context* ctx = nullptr;
  uint32_t n = 0, P = 0;
  int dtype = QPE_C64;
  size_t esz = 8;
  uint64_t N = 0;
  std::vector<const qpe_program*> progs;
  std::vector<uint64_t> ld, off;  // per instance: block size, element offset of its register
  DevBuf regs, works, probs, partial, tw;
  uint32_t max_qift_grid = 1;
  std::deque<BatchClass> classes;  // stable addresses: BatchClass owns device buffers
  uint64_t touches_per_run = 0;
  uint32_t launches_per_run = 0;
  cudaGraphExec_t exec = nullptr;
  cudaStream_t side = nullptr;
  ~qpe_batch() {
    if (exec) cudaGraphExecDestroy(exec);
    if (side) cudaStreamDestroy(side);
  }
};

namespace {

void plan_class(qpe_batch* b, BatchClass& c) {
  const HostProgram& hp = c.shape->hp;
  c.plans.clear();
  for (uint32_t sw = 0; sw < hp.steps * hp.order; ++sw) {
    const bool rev = hp.order == 2 && (sw & 1);
    for (size_t pj = 0; pj < hp.passes.size(); ++pj) {
      const Pass& pass = hp.passes[rev ? hp.passes.size() - 1 - pj : pj];
      PassLaunch pl = plan_pass_geometry(c.shape, b->esz, b->ctx->smem_optin, pass);
      if (pass.type == PASS_COL && c.W) pl.W = c.W;
      const size_t stage = pass_stage_elems(pass, pl.Ca, pl.Cb, pl.W) * b->esz;
      // wpc == 0 selects one tile per CTA (its threads split every term's entries)
      pl.cta_tile = c.wpc == 0 ? kCtaTileThreads : 0u;
      uint32_t wpc = c.wpc ? c.wpc : kCtaTileThreads / 32;
      while (!pl.cta_tile && wpc > 1 && stage * wpc > b->ctx->smem_optin) --wpc;
      pl.warps_per_cta = wpc;
      if (pl.img && pass_smem_bytes(pl, b->esz) > b->ctx->smem_optin) {  // the image only where it fits
        pl.img = nullptr;
        pl.img_words = 0;
      }
      const uint64_t ntiles = pass.type == PASS_COL ? (hp.Cb + pl.W - 1) / pl.W
                                                    : (pass.type == PASS_ROW ? hp.Ca : pass.mixcount);
      const uint32_t slots = pl.cta_tile ? 1u : wpc;
      uint64_t grid = (ntiles * c.members.size() + slots - 1) / slots;
      const uint64_t cap = (uint64_t)b->ctx->num_sms * 16;
      pl.grid = (uint32_t)std::max<uint64_t>(1, std::min(grid, cap));
      pl.rev = rev ? 1u : 0u;
      pl.exact = b->dtype == QPE_C128 ? 1u : 0u;
      pl.works = c.works_ptr.as<void*>();
      pl.icoef = c.icoef.as<double2>();
      pl.nmem = (uint32_t)c.members.size();
      pl.nops = (uint32_t)hp.ops.size();
      c.plans.push_back(pl);
    }
  }
}

size_t plans_smem(const qpe_batch* b, const BatchClass& c) {
  size_t m = 48 * 1024;
  for (const PassLaunch& pl : c.plans) m = std::max(m, pass_smem_bytes(pl, b->esz));
  return m;
}

void launch_power(qpe_batch* b, BatchClass& c, cudaStream_t s) {
  for (const PassLaunch& pl : c.plans) QPE_CK(launch_pass(pl, b->dtype, s));
}

// Times one power of each tile shape on the class's first power and keeps the best.
void tune_class(qpe_batch* b, BatchClass& c) {
  cudaStream_t s = b->ctx->stream;
  cudaEvent_t e0, e1;
  QPE_CK(cudaEventCreate(&e0));
  QPE_CK(cudaEventCreate(&e1));
  float best = 1e30f;
  uint32_t bw = 1, bwpc = 4;
  for (uint32_t W : {1u, 2u, 4u, 8u}) {
    if ((uint64_t)W * 2 > c.shape->hp.Cb && W > 1) continue;
    for (uint32_t wpc : {0u, 2u, 4u, 8u}) {  // 0: one tile per CTA
      c.W = W;
      c.wpc = wpc;
      plan_class(b, c);
      QPE_CK(configure_pass_kernels(b->dtype, plans_smem(b, c)));
      QPE_CK(launch_load_batch(c.works_ptr.as<void*>(), c.states_ptr.as<void*>(), (uint32_t)c.shape->hp.Ca,
                               (uint32_t)c.shape->hp.Cb, 0, (uint32_t)c.members.size(), b->dtype, s));
      launch_power(b, c, s);  // warm-up
      QPE_CK(cudaEventRecord(e0, s));
      launch_power(b, c, s);
      QPE_CK(cudaEventRecord(e1, s));
      QPE_CK(cudaEventSynchronize(e1));
      float ms = 0;
      QPE_CK(cudaEventElapsedTime(&ms, e0, e1));
      if (ms < best) {
        best = ms;
        bw = W;
        bwpc = wpc;
      }
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  c.W = bw;
  c.wpc = bwpc;
  c.tuned_ms = best;
  plan_class(b, c);
}

void build_graph(qpe_batch* b) {
  cudaStream_t s = b->ctx->stream;
  size_t smem = 48 * 1024;
  for (BatchClass& c : b->classes) smem = std::max(smem, plans_smem(b, c));
  QPE_CK(configure_pass_kernels(b->dtype, smem));
  // One shared-memory limit for every instance's QIFT: the largest tile's.
  uint32_t T = 1, grid = 1;
  size_t qsmem = 0;
  for (uint32_t i = 0; i < b->n; ++i) {
    qift_geometry(b->P, b->ld[i], b->dtype, b->ctx->num_sms, b->ctx->smem_optin, T, grid);
    qsmem = std::max(qsmem, qift_smem_bytes(b->P, T, b->dtype));
  }
  QPE_CK(configure_qift_kernels(b->dtype, qsmem));
  const int last = (int)b->N;
  b->launches_per_run = 0;
  QPE_CK(cudaStreamBeginCapture(s, cudaStreamCaptureModeRelaxed));
  cudaError_t err = cudaSuccess;
  cudaGraph_t g = nullptr;
  std::vector<cudaGraphNode_t> loops;
  try {
    // Working blocks <- block 0; power counter <- 1.
    for (BatchClass& c : b->classes) {
      QPE_CK(launch_load_batch(c.works_ptr.as<void*>(), c.states_ptr.as<void*>(), (uint32_t)c.shape->hp.Ca,
                               (uint32_t)c.shape->hp.Cb, 0, (uint32_t)c.members.size(), b->dtype, s));
      QPE_CK(cudaMemsetAsync(c.dk.p, 0, sizeof(int), s));
      b->launches_per_run += 1;
    }
    cudaStreamCaptureStatus cs;
    cudaGraph_t cg = nullptr;
    const cudaGraphNode_t* deps = nullptr;
    size_t ndeps = 0;
    QPE_CK(cudaStreamGetCaptureInfo(s, &cs, nullptr, &cg, &deps, nullptr, &ndeps));
    std::vector<cudaGraphNode_t> root(deps, deps + ndeps);
    for (BatchClass& c : b->classes) {
      // The counter holds k - 1 on entry to the body; the body advances it to k,
      // runs power k, writes block k, and continues while k + 1 < 2^P.
      cudaGraphConditionalHandle h;
      QPE_CK(cudaGraphConditionalHandleCreate(&h, cg, 1, cudaGraphCondAssignDefault));
      alignas(cudaGraphNodeParams) unsigned char np_raw[sizeof(cudaGraphNodeParams)] = {};
      cudaGraphNodeParams& np = *reinterpret_cast<cudaGraphNodeParams*>(np_raw);
      np.type = cudaGraphNodeTypeConditional;
      np.conditional.handle = h;
      np.conditional.type = cudaGraphCondTypeWhile;
      np.conditional.size = 1;
      cudaGraphNode_t node;
      QPE_CK(cudaGraphAddNode(&node, cg, root.data(), nullptr, root.size(), &np));
      loops.push_back(node);
      cudaGraph_t body = np.conditional.phGraph_out[0];
      QPE_CK(cudaStreamBeginCaptureToGraph(b->side, body, nullptr, nullptr, 0, cudaStreamCaptureModeRelaxed));
      QPE_CK(launch_advance(c.dk.as<int>(), b->side));  // k - 1 -> k
      launch_power(b, c, b->side);
      QPE_CK(launch_snapshot_batch(c.works_ptr.as<void*>(), c.states_ptr.as<void*>(), (uint32_t)c.shape->hp.Ca,
                                   (uint32_t)c.shape->hp.Cb, c.dk.as<int>(), (uint32_t)c.members.size(), b->dtype,
                                   b->side));
      QPE_CK(launch_continue_while(c.dk.as<int>(), last, h, b->side));
      cudaGraph_t body_out = nullptr;
      QPE_CK(cudaStreamEndCapture(b->side, &body_out));
      b->launches_per_run += (uint32_t)((c.plans.size() + 3) * (b->N - 1));
    }
    QPE_CK(cudaStreamUpdateCaptureDependencies(s, loops.data(), nullptr, loops.size(), cudaStreamSetCaptureDependencies));
    // QIFT and histogram of every instance.
    const double norm = std::sqrt((double)b->N);
    for (uint32_t i = 0; i < b->n; ++i) {
      qift_geometry(b->P, b->ld[i], b->dtype, b->ctx->num_sms, b->ctx->smem_optin, T, grid);
      QPE_CK(launch_qift(b->regs.as<char>() + b->off[i] * b->esz, b->ld[i], b->P, b->tw.p, norm,
                         b->partial.as<double>(), grid, T, b->dtype, s));
      QPE_CK(launch_reduce_partials(b->partial.as<double>(), grid, (uint32_t)b->N, b->probs.as<double>() + i * b->N, s));
      b->launches_per_run += 2;
    }
  } catch (...) {
    cudaStreamEndCapture(s, &g);
    if (g) cudaGraphDestroy(g);
    throw;
  }
  err = cudaStreamEndCapture(s, &g);
  QPE_CK(err);
  cudaGraphExec_t ge = nullptr;
  err = cudaGraphInstantiate(&ge, g, 0);
  cudaGraphDestroy(g);
  QPE_CK(err);
  if (b->exec) cudaGraphExecDestroy(b->exec);
  b->exec = ge;
}

}  // namespace

extern "C" {

int qpe_batch_create(qpe_context* ctx, uint32_t n, const qpe_program* const* programs, uint32_t P, int dtype,
                     qpe_batch** out) {
  return guard([&] {
    if (!ctx || !out || (n && !programs)) throw Error(QPE_ERR_INVALID, "null argument");
    *out = nullptr;
    if (n == 0) throw Error(QPE_ERR_INVALID, "empty batch");
    if (P == 0 || P > 13) throw Error(QPE_ERR_UNSUPPORTED, "precision must be in 1..13");
    if (dtype != QPE_C128 && dtype != QPE_C64) throw Error(QPE_ERR_INVALID, "unknown dtype");
    QPE_CK(cudaSetDevice(ctx->device));
    auto b = new qpe_batch();
    try {
      b->ctx = ctx;
      b->n = n;
      b->P = P;
      b->dtype = dtype;
      b->esz = dtype == QPE_C128 ? 16 : 8;
      b->N = 1ull << P;
      uint64_t total = 0, work_total = 0;
      for (uint32_t i = 0; i < n; ++i) {
        const qpe_program* pr = programs[i];
        if (!pr || pr->ctx != ctx) throw Error(QPE_ERR_INVALID, "program missing or from another context");
        b->progs.push_back(pr);
        b->ld.push_back(pr->hp.Ca * pr->hp.Cb);
        b->off.push_back(total);
        total += b->N * b->ld.back();
        work_total += (b->ld.back() + 1) / 2 * 2;  // padded to 16 bytes (see work_off)
        b->touches_per_run += pr->hp.touches_per_power * (b->N - 1);
      }
      b->regs.alloc(total * b->esz);
      QPE_CK(cudaMemset(b->regs.p, 0, total * b->esz));
      b->works.alloc(work_total * b->esz);
      b->probs.alloc(n * b->N * sizeof(double));
      uint32_t T = 1, grid = 1;
      for (uint32_t i = 0; i < n; ++i) {
        qift_geometry(P, b->ld[i], dtype, ctx->num_sms, ctx->smem_optin, T, grid);
        b->max_qift_grid = std::max(b->max_qift_grid, grid);
      }
      b->partial.alloc((size_t)b->max_qift_grid * b->N * sizeof(double));
      state_twiddles(P, dtype, b->tw);
      // Classes of identical structure; members ordered by size, largest first.
      std::vector<uint32_t> order(n);
      std::iota(order.begin(), order.end(), 0u);
      std::stable_sort(order.begin(), order.end(), [&](uint32_t x, uint32_t y) {
        return b->progs[x]->hp.touches_per_power > b->progs[y]->hp.touches_per_power;
      });
      std::vector<uint64_t> work_off(n);
      {
        // every working block starts on a 16-byte boundary (bulk copies of its columns)
        const uint64_t align = 16 / b->esz;
        uint64_t o = 0;
        for (uint32_t i = 0; i < n; ++i) {
          work_off[i] = o;
          o += (b->ld[i] + align - 1) / align * align;
        }
      }
      for (uint32_t i : order) {
        const HostProgram& hp = b->progs[i]->hp;
        for (const DevOp& d : hp.ops)
          if (d.gen != OP_INLINE) throw Error(QPE_ERR_UNSUPPORTED, "batched terms need m00 real and m01 imaginary");
        BatchClass* cls = nullptr;
        for (BatchClass& c : b->classes)
          if (same_structure(c.shape->hp, hp)) cls = &c;
        if (!cls) {
          b->classes.emplace_back();
          cls = &b->classes.back();
          cls->shape = b->progs[i];
          cls->ld = b->ld[i];
        }
        cls->members.push_back(i);
      }
      for (BatchClass& c : b->classes) {
        const size_t m = c.members.size(), nops = c.shape->hp.ops.size();
        std::vector<double> co(2 * m * std::max<size_t>(nops, 1));
        std::vector<void*> wp(m), sp(m);
        for (size_t k = 0; k < m; ++k) {
          const uint32_t i = c.members[k];
          const HostProgram& hp = b->progs[i]->hp;
          for (size_t o = 0; o < nops; ++o) {
            co[2 * (k * nops + o)] = hp.ops[o].c0;
            co[2 * (k * nops + o) + 1] = hp.ops[o].c1;
          }
          wp[k] = b->works.as<char>() + work_off[i] * b->esz;
          sp[k] = b->regs.as<char>() + b->off[i] * b->esz;
        }
        c.icoef.alloc(co.size() * sizeof(double));
        QPE_CK(cudaMemcpy(c.icoef.p, co.data(), co.size() * sizeof(double), cudaMemcpyHostToDevice));
        c.works_ptr.alloc(m * sizeof(void*));
        c.states_ptr.alloc(m * sizeof(void*));
        QPE_CK(cudaMemcpy(c.works_ptr.p, wp.data(), m * sizeof(void*), cudaMemcpyHostToDevice));
        QPE_CK(cudaMemcpy(c.states_ptr.p, sp.data(), m * sizeof(void*), cudaMemcpyHostToDevice));
        c.dk.alloc(sizeof(int));
        plan_class(b, c);
      }
      QPE_CK(cudaStreamCreateWithFlags(&b->side, cudaStreamNonBlocking));
    } catch (...) {
      delete b;
      throw;
    }
    *out = b;
  });
}

int qpe_batch_destroy(qpe_batch* b) {
  if (!b) return QPE_OK;
  cudaSetDevice(b->ctx->device);
  cudaStreamSynchronize(b->ctx->stream);
  delete b;
  return QPE_OK;
}

int qpe_batch_upload(qpe_batch* b, uint32_t i, const void* host, uint64_t first, uint64_t count) {
  return guard([&] {
    if (!b || (count && !host)) throw Error(QPE_ERR_INVALID, "null argument");
    if (i >= b->n) throw Error(QPE_ERR_INVALID, "instance out of range");
    const uint64_t size = b->N * b->ld[i];
    if (first > size || count > size - first) throw Error(QPE_ERR_INVALID, "range outside the register");
    QPE_CK(cudaSetDevice(b->ctx->device));
    QPE_CK(cudaMemcpyAsync(b->regs.as<char>() + (b->off[i] + first) * b->esz, host, count * b->esz,
                           cudaMemcpyHostToDevice, b->ctx->stream));
    QPE_CK(cudaStreamSynchronize(b->ctx->stream));
  });
}

int qpe_batch_download(qpe_batch* b, uint32_t i, void* host, uint64_t first, uint64_t count) {
  return guard([&] {
    if (!b || (count && !host)) throw Error(QPE_ERR_INVALID, "null argument");
    if (i >= b->n) throw Error(QPE_ERR_INVALID, "instance out of range");
    const uint64_t size = b->N * b->ld[i];
    if (first > size || count > size - first) throw Error(QPE_ERR_INVALID, "range outside the register");
    QPE_CK(cudaSetDevice(b->ctx->device));
    QPE_CK(cudaMemcpyAsync(host, b->regs.as<char>() + (b->off[i] + first) * b->esz, count * b->esz,
                           cudaMemcpyDeviceToHost, b->ctx->stream));
    QPE_CK(cudaStreamSynchronize(b->ctx->stream));
    check_device_error(b->ctx);
  });
}

int qpe_batch_tune(qpe_batch* b) {
  return guard([&] {
    if (!b) throw Error(QPE_ERR_INVALID, "null batch");
    QPE_CK(cudaSetDevice(b->ctx->device));
    for (BatchClass& c : b->classes) tune_class(b, c);
    if (b->exec) {
      cudaGraphExecDestroy(b->exec);
      b->exec = nullptr;
    }
  });
}

int qpe_batch_run(qpe_batch* b, int synchronize) {
  return guard([&] {
    if (!b) throw Error(QPE_ERR_INVALID, "null batch");
    QPE_CK(cudaSetDevice(b->ctx->device));
    if (!b->exec) build_graph(b);
    QPE_CK(cudaGraphLaunch(b->exec, b->ctx->stream));
    if (synchronize) {
      QPE_CK(cudaStreamSynchronize(b->ctx->stream));
      check_device_error(b->ctx);
    }
  });
}

int qpe_batch_phase_probs(qpe_batch* b, uint32_t i, double* probs) {
  return guard([&] {
    if (!b || !probs) throw Error(QPE_ERR_INVALID, "null argument");
    if (i >= b->n) throw Error(QPE_ERR_INVALID, "instance out of range");
    QPE_CK(cudaSetDevice(b->ctx->device));
    QPE_CK(cudaMemcpyAsync(probs, b->probs.as<double>() + i * b->N, b->N * sizeof(double), cudaMemcpyDeviceToHost,
                           b->ctx->stream));
    QPE_CK(cudaStreamSynchronize(b->ctx->stream));
    check_device_error(b->ctx);
  });
}

int qpe_batch_get_info(const qpe_batch* b, qpe_batch_info* info) {
  if (!b || !info) return fail(QPE_ERR_INVALID, "null argument");
  std::memset(info, 0, sizeof(*info));
  info->instances = b->n;
  info->classes = (uint32_t)b->classes.size();
  info->touches_per_run = b->touches_per_run;
  info->launches_per_run = b->launches_per_run;
  uint64_t amps = 0;
  for (uint32_t i = 0; i < b->n; ++i) amps += b->N * b->ld[i];
  info->amplitudes = amps;
  return QPE_OK;
}

int qpe_batch_class_info(const qpe_batch* b, uint32_t cls, qpe_batch_class* out) {
  if (!b || !out) return fail(QPE_ERR_INVALID, "null argument");
  if (cls >= b->classes.size()) return fail(QPE_ERR_INVALID, "class index out of range");
  const BatchClass& c = b->classes[cls];
  const HostProgram& hp = c.shape->hp;
  std::memset(out, 0, sizeof(*out));
  out->num_orbitals = hp.M;
  out->n_alpha = hp.na;
  out->n_beta = hp.nb;
  out->members = (uint32_t)c.members.size();
  out->touches_per_power = hp.touches_per_power * c.members.size();
  out->ms_per_power = c.tuned_ms;
  out->tile_lines = c.W;
  out->warps_per_cta = c.wpc;
  return QPE_OK;
}

}  // extern "C"
