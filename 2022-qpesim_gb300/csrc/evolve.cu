// evolve.cu - tile-pass kernels of the Trotterized evolution.
//
// Each launch runs one pass (program.h) over the working block. A warp owns one
// tile at a time: it gathers the tile's lines from the working block into a
// warp-private shared-memory stage, applies the pass's term applications in order
// (__syncwarp between terms), and scatters the tile back. Tiles of one pass are
// disjoint and closed under the pass's terms, so warps never wait on each other.
//
// The pair update is the reference's updateStateVector
// (cpp/time_evolution_over_terms.hpp:565-589): l' = l*m00 + r*m01, r' = l*m01 + r*m00.
// For complex128 in exact mode every product and sum is rounded separately in the
// order std::complex<double> arithmetic uses, so the result is bit-identical to the
// reference compiled without floating-point contraction. Terms whose matrices have
// a real m00 and an imaginary m01 (every pq / pqqr / pqrs term the Hamiltonian
// getters produce) skip the products with exact zeros, which changes no bit.
#include <cuda_runtime.h>

#include <map>
#include <mutex>
#include <type_traits>
#include <stdint.h>

#include "kernels.h"
#include "tile_ops.cuh"

namespace qpe {

// One element from global to shared memory without passing through registers
// (cp.async, 8 or 16 bytes; the caller commits and waits).
template <typename C2>
__device__ __forceinline__ void async_copy(C2* dst, const C2* src) {
  const uint32_t d = static_cast<uint32_t>(__cvta_generic_to_shared(dst));
  if constexpr (sizeof(C2) == 16)
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(d), "l"(src) : "memory");
  else
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8;" ::"r"(d), "l"(src) : "memory");
}

// Bulk copies between global and shared memory (cp.async.bulk). A load
// completes on an mbarrier of this CTA (transaction bytes); a store is tracked
// by the issuing thread's bulk async-group. Addresses and sizes are multiples of
// 16 bytes.
__device__ __forceinline__ void bulk_load(void* sdst, const void* gsrc, uint32_t bytes, uint32_t bar) {
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                   static_cast<uint32_t>(__cvta_generic_to_shared(sdst))),
               "l"(gsrc), "r"(bytes), "r"(bar)
               : "memory");
}
__device__ __forceinline__ void bulk_store(void* gdst, const void* ssrc, uint32_t bytes) {
  asm volatile("cp.async.bulk.global.shared::cta.bulk_group [%0], [%1], %2;" ::"l"(gdst),
               "r"(static_cast<uint32_t>(__cvta_generic_to_shared(ssrc))), "r"(bytes)
               : "memory");
}
__device__ __forceinline__ void mbar_init1(uint32_t bar) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(bar) : "memory");
}
__device__ __forceinline__ void mbar_arrive_tx(uint32_t bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
}
// Bounded wait for the phase of the given parity (about 2^24 polls, far longer
// than any copy of a tile takes).
__device__ __forceinline__ bool mbar_wait_bounded(uint32_t bar, uint32_t parity) {
  for (uint32_t i = 0; i < (1u << 24); ++i) {
    uint32_t done;
    asm volatile(
        "{\n"
        ".reg .pred p;\n"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
        "selp.u32 %0, 1, 0, p;\n"
        "}\n"
        : "=r"(done)
        : "r"(bar), "r"(parity)
        : "memory");
    if (done) return true;
  }
  return false;
}

// One pass. PT selects the tile geometry; the stage holds a tile by lines:
//   PASS_COL: tile = W consecutive columns, stage[w * Ca + e] = block[e][b0 + w]
//   PASS_ROW: tile = one row,               stage[e]          = block[a][e]
//   PASS_MIX: tile = columns (b01, b10),    stage[w * Ca + e] = block[e][w ? b10 : b01]
// The working block is stored by columns, so a COL or MIX tile's lines are
// contiguous runs of it. With pl.bulk they move as whole runs by bulk copies:
// one thread of the tile issues the loads (the W columns of a COL tile are one
// run; a MIX tile's two columns are two), every thread of the tile waits on the
// tile's mbarrier, and after the updates the same thread writes the runs back
// with bulk stores. Otherwise every thread copies elements with cp.async.
//
// CT: a whole CTA shares one tile (its threads split each term's entries, a CTA
// barrier between terms); otherwise every warp owns its own tile.
template <typename R, class A, int PT, bool CT>
__global__ void k_pass(PassLaunch pl) {
  using C2 = typename Cx<R>::T;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ __align__(8) uint64_t bars[CT ? 1 : 32];  // one mbarrier per tile slot (bulk copies)
  __shared__ __align__(8) uint64_t imgbar;              // the pass image's bulk copy
  const uint32_t lane = CT ? threadIdx.x : (threadIdx.x & 31);  // thread index within the tile
  const uint32_t tpt = CT ? blockDim.x : 32u;                    // threads per tile
  const uint32_t warp = CT ? 0u : (threadIdx.x >> 5);            // tile slot within the CTA
  const uint32_t wpc = CT ? 1u : (blockDim.x >> 5);              // tile slots per CTA
  using Sync = typename std::conditional<CT, CtaSync, WarpSync>::type;
  const uint32_t Ca = pl.Ca, Cb = pl.Cb;
  const uint32_t W = (PT == PASS_COL) ? pl.W : (PT == PASS_ROW ? 1u : 2u);
  const uint32_t L = (PT == PASS_ROW) ? Cb : Ca;
  const uint32_t logW = __ffs(W) - 1;
  C2* __restrict__ st = reinterpret_cast<C2*>(smem_raw) + (size_t)warp * L * W;
  const uint32_t* __restrict__ pool = pl.pool;
  const bool bulk = PT != PASS_ROW && pl.bulk != 0;
  const uint32_t bar = static_cast<uint32_t>(__cvta_generic_to_shared(&bars[warp]));
  // A MIX pass's image (descriptors and tables) in shared memory behind the
  // stages, brought in once per CTA by one bulk copy.
  const bool image = PT == PASS_MIX && bulk && pl.img != nullptr;
  uint32_t* img_s = reinterpret_cast<uint32_t*>(reinterpret_cast<C2*>(smem_raw) + (size_t)wpc * L * W);
  const uint32_t ibar = static_cast<uint32_t>(__cvta_generic_to_shared(&imgbar));
  if (bulk) {
    if (lane == 0) {
      mbar_init1(bar);
      if (image && threadIdx.x == 0) mbar_init1(ibar);
      asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();
    if (image && threadIdx.x == 0) {
      mbar_arrive_tx(ibar, pl.img_words * 4u);
      bulk_load(img_s, pl.img, pl.img_words * 4u, ibar);
    }
  }
  bool image_ready = !image;
  uint32_t phase = 0;
  uint32_t ntiles;
  if (PT == PASS_COL) ntiles = (Cb + W - 1) >> logW;
  else if (PT == PASS_ROW) ntiles = Ca;
  else ntiles = pl.pass.mixcount;
  const uint32_t nmem = pl.nmem ? pl.nmem : 1u;
  for (uint32_t gt = blockIdx.x * wpc + warp; gt < ntiles * nmem; gt += gridDim.x * wpc) {
    const uint32_t mem = gt / ntiles, tile = gt - mem * ntiles;
    C2* __restrict__ blk = reinterpret_cast<C2*>(pl.works ? pl.works[mem] : pl.work);
    const double2* icoef = pl.icoef ? pl.icoef + (size_t)mem * pl.nops : nullptr;
    uint32_t b0 = 0, b01 = 0, b10 = 0, parb = 0, row = 0;
    if (PT == PASS_COL) b0 = tile << logW;
    if (PT == PASS_ROW) row = tile;
    if (PT == PASS_MIX) {
      const uint2 x = __ldg(reinterpret_cast<const uint2*>(pool + pl.pass.mixtab) + tile);
      b01 = x.x & 0x7fffffffu;
      b10 = x.y;
      parb = x.x >> 31;
    }
    const uint32_t nl = (PT == PASS_COL) ? min(W, Cb - b0) : W;  // valid lines
    // The tile's runs of the working block: line w of the stage is Ca (or, for a
    // row, Cb) elements from column col(w) on (a row: strided, element-wise).
    auto col = [&](uint32_t w) -> uint32_t { return PT == PASS_COL ? b0 + w : (w ? b10 : b01); };
    if (bulk) {
      if (lane == 0) {
        const uint32_t bytes = Ca * (uint32_t)sizeof(C2);
        mbar_arrive_tx(bar, nl * bytes);
        if (PT == PASS_COL) {
          bulk_load(st, blk + (uint64_t)b0 * Ca, nl * bytes, bar);
        } else {
          bulk_load(st, blk + (uint64_t)b01 * Ca, bytes, bar);
          bulk_load(st + Ca, blk + (uint64_t)b10 * Ca, bytes, bar);
        }
      }
      bool ok = mbar_wait_bounded(bar, phase);
      if (!image_ready) ok = mbar_wait_bounded(ibar, 0) && ok;  // the image, before the first tile's terms
      ok = CT ? (__syncthreads_and(ok) != 0) : (__all_sync(0xffffffffu, ok) != 0);  // one verdict per tile
      if (!ok) {
        // the copies did not complete: record it, give the copies in flight one
        // more bounded wait, and stop (the pass's results are invalid)
        if (lane == 0) {
          atomicOr(pl.err, kPassErrWait);
          mbar_wait_bounded(bar, phase);
          if (!image_ready) mbar_wait_bounded(ibar, 0);
        }
        break;
      }
      phase ^= 1u;
      image_ready = true;
    } else {
      // all of the tile's element copies in flight at once (cp.async), so the
      // tile pays the L2 latency once rather than once per element
      if (PT == PASS_ROW) {
        for (uint32_t e = lane; e < L; e += tpt) async_copy(st + e, blk + (uint64_t)e * Ca + row);
      } else {
        for (uint32_t w = 0; w < nl; ++w)
          for (uint32_t e = lane; e < Ca; e += tpt) async_copy(st + w * Ca + e, blk + (uint64_t)col(w) * Ca + e);
      }
      asm volatile("cp.async.commit_group;\ncp.async.wait_group 0;" ::: "memory");
    }
    Sync()();
    if (PT == PASS_MIX && image) {
      // descriptors and tables from the image: terms 0 .. n - 1 of the pass, the
      // batch members' coefficients at the pass's own op indices
      chunked_mix_ops<R, A, false>(reinterpret_cast<const DevOp*>(img_s), pl.coef, img_s, 0u,
                                   pl.pass.op1 - pl.pass.op0, pl.rev != 0, lane, tpt, true, parb,
                                   [&](uint32_t a) -> C2& { return st[a]; },
                                   [&](uint32_t a) -> C2& { return st[Ca + a]; },
                                   icoef ? icoef + pl.pass.op0 : nullptr, Sync());
    } else if (PT == PASS_MIX) {
      chunked_mix_ops<R, A>(pl.ops, pl.coef, pool, pl.pass.op0, pl.pass.op1, pl.rev != 0, lane, tpt, true, parb,
                            [&](uint32_t a) -> C2& { return st[a]; }, [&](uint32_t a) -> C2& { return st[Ca + a]; },
                            icoef, Sync());
    } else {
      // Lane l owns line l % W and walks entries l / W, l / W + 32 / W, ...
      const uint32_t w = lane & (W - 1);
      const bool active = w < nl;
      const uint32_t line = (PT == PASS_COL) ? b0 + w : row;
      const uint32_t lstr = active ? __ldg(((PT == PASS_COL) ? pl.strB : pl.strA) + line) : 0u;
      chunked_line_ops<R, A>(pl.ops, pl.coef, pool, pl.pass.op0, pl.pass.op1, pl.rev != 0, L, lane >> logW,
                             tpt >> logW, active, lstr, [&](uint32_t e) -> C2& { return st[w * L + e]; }, icoef,
                             Sync());
    }
    if (bulk) {
      // the updates (generic proxy) must be visible to the bulk copy (async proxy)
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
      Sync()();
      if (lane == 0) {
        const uint32_t bytes = Ca * (uint32_t)sizeof(C2);
        if (PT == PASS_COL) {
          bulk_store(blk + (uint64_t)b0 * Ca, st, nl * bytes);
        } else {
          bulk_store(blk + (uint64_t)b01 * Ca, st, bytes);
          bulk_store(blk + (uint64_t)b10 * Ca, st + Ca, bytes);
        }
        asm volatile("cp.async.bulk.commit_group;" ::: "memory");
        // the stage is read before the next tile's loads overwrite it
        asm volatile("cp.async.bulk.wait_group.read 0;" ::: "memory");
      }
    } else if (PT == PASS_ROW) {
      for (uint32_t e = lane; e < L; e += tpt) blk[(uint64_t)e * Ca + row] = st[e];
    } else {
      for (uint32_t w = 0; w < nl; ++w)
        for (uint32_t e = lane; e < Ca; e += tpt) blk[(uint64_t)col(w) * Ca + e] = st[w * Ca + e];
    }
    Sync()();
  }
  // the bulk stores are complete (in global memory) before the CTA exits
  if (bulk && lane == 0) asm volatile("cp.async.bulk.wait_group 0;" ::: "memory");
}

size_t pass_stage_elems(const Pass& pass, uint32_t Ca, uint32_t Cb, uint32_t W) {
  if (pass.type == PASS_COL) return (size_t)Ca * W;
  if (pass.type == PASS_ROW) return (size_t)Cb;
  return (size_t)Ca * 2;
}

size_t pass_smem_bytes(const PassLaunch& pl, size_t esz) {
  return pass_stage_elems(pl.pass, pl.Ca, pl.Cb, pl.W) * esz * (pl.cta_tile ? 1 : pl.warps_per_cta) +
         (pl.img ? (size_t)pl.img_words * 4 : 0);
}

// dst[segs[i].dst + k] = src[segs[i].src + k], k < segs[i].words: the tables of
// the pass images, one CTA per segment.
__global__ void k_copy_segments(const uint32_t* __restrict__ src, uint32_t* __restrict__ dst,
                                const PassImageSeg* __restrict__ segs, uint32_t n) {
  for (uint32_t i = blockIdx.x; i < n; i += gridDim.x) {
    const PassImageSeg g = segs[i];
    for (uint32_t k = threadIdx.x; k < g.words; k += blockDim.x) dst[g.dst + k] = src[g.src + k];
  }
}

cudaError_t launch_copy_segments(const uint32_t* src, uint32_t* dst, const PassImageSeg* segs, uint32_t n,
                                 cudaStream_t s) {
  if (n == 0) return cudaSuccess;
  k_copy_segments<<<n < 4096 ? n : 4096, 128, 0, s>>>(src, dst, segs, n);
  return cudaGetLastError();
}

template <typename R, class A, bool CT>
static cudaError_t launch_ct(const PassLaunch& pl, cudaStream_t s) {
  using C2 = typename Cx<R>::T;
  const size_t smem = pass_smem_bytes(pl, sizeof(C2));
  const dim3 block(CT ? pl.cta_tile : 32 * pl.warps_per_cta);
  switch (pl.pass.type) {
    case PASS_COL: k_pass<R, A, PASS_COL, CT><<<pl.grid, block, smem, s>>>(pl); break;
    case PASS_ROW: k_pass<R, A, PASS_ROW, CT><<<pl.grid, block, smem, s>>>(pl); break;
    default: k_pass<R, A, PASS_MIX, CT><<<pl.grid, block, smem, s>>>(pl); break;
  }
  return cudaGetLastError();
}

template <typename R, class A>
static cudaError_t launch_typed(const PassLaunch& pl, cudaStream_t s) {
  return pl.cta_tile ? launch_ct<R, A, true>(pl, s) : launch_ct<R, A, false>(pl, s);
}

cudaError_t launch_pass(const PassLaunch& pl, int dtype, cudaStream_t s) {
  if (dtype == QPE_C128) {
    if (pl.exact) return launch_typed<double, ExactD>(pl, s);
    return launch_typed<double, Fast<double>>(pl, s);
  }
  return launch_typed<float, Fast<float>>(pl, s);
}

template <typename R, class A, bool CT>
static cudaError_t configure_ct(size_t smem) {
  cudaError_t e;
  if ((e = cudaFuncSetAttribute(k_pass<R, A, PASS_COL, CT>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem)))
    return e;
  if ((e = cudaFuncSetAttribute(k_pass<R, A, PASS_ROW, CT>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem)))
    return e;
  return cudaFuncSetAttribute(k_pass<R, A, PASS_MIX, CT>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
}

template <typename R, class A>
static cudaError_t configure_typed(size_t smem) {
  cudaError_t e = configure_ct<R, A, false>(smem);
  if (e) return e;
  return configure_ct<R, A, true>(smem);
}

// The shared-memory limit is a property of the kernel, not of one launch or one
// captured graph, so it only ever grows: a later, smaller request must not break
// the launches (and graphs) planned for a larger one.
cudaError_t configure_pass_kernels(int dtype, size_t smem) {
  static std::mutex mu;
  static std::map<std::pair<int, int>, size_t> granted;  // (device, dtype) -> bytes
  int dev = 0;
  cudaGetDevice(&dev);
  std::lock_guard<std::mutex> lock(mu);
  size_t& g = granted[{dev, dtype}];
  if (smem <= g) return cudaSuccess;
  cudaError_t e;
  if (dtype == QPE_C128) {
    e = configure_typed<double, ExactD>(smem);
    if (e == cudaSuccess) e = configure_typed<double, Fast<double>>(smem);
  } else {
    e = configure_typed<float, Fast<float>>(smem);
  }
  if (e == cudaSuccess) g = smem;
  return e;
}

// The working block is stored by columns (element (a, b) at b * Ca + a), so that
// a column, the tile of COL passes and each half of a MIX tile, is contiguous
// and its gather and scatter are coalesced. The register keeps the reference's
// row-major blocks (a * Cb + b); loads and snapshots transpose in 32 x 32 tiles
// through shared memory.
//
// dst (C x R, row-major) = transpose of src (R x C, row-major); blockIdx.z picks
// member z of a batch when the pointer arrays are given.
template <typename C2>
__device__ __forceinline__ void transpose_tile(const C2* __restrict__ src, C2* __restrict__ dst, uint32_t R,
                                               uint32_t C) {
  __shared__ C2 tile[32][33];
  const uint32_t c0 = blockIdx.x * 32, r0 = blockIdx.y * 32;
  for (uint32_t y = threadIdx.y; y < 32; y += blockDim.y) {
    const uint32_t r = r0 + y, c = c0 + threadIdx.x;
    if (r < R && c < C) tile[y][threadIdx.x] = src[(uint64_t)r * C + c];
  }
  __syncthreads();
  for (uint32_t y = threadIdx.y; y < 32; y += blockDim.y) {
    const uint32_t c = c0 + y, r = r0 + threadIdx.x;
    if (r < R && c < C) dst[(uint64_t)c * R + r] = tile[threadIdx.x][y];
  }
}

// Snapshot of the working block into block *d_k of the state
// (std::copy_n of :130-132, taken after the power instead of before).
template <typename C2>
__global__ void k_snapshot(const C2* __restrict__ work, C2* __restrict__ state, uint32_t Ca, uint32_t Cb,
                           const int* d_k) {
  transpose_tile(work, state + (uint64_t)*d_k * Ca * Cb, Cb, Ca);
}

// Block `block` of the state into the working block.
template <typename C2>
__global__ void k_load(C2* __restrict__ work, const C2* __restrict__ state, uint32_t Ca, uint32_t Cb, uint32_t block) {
  transpose_tile(state + (uint64_t)block * Ca * Cb, work, Ca, Cb);
}

__global__ void k_advance(int* d_k) { *d_k += 1; }

template <typename C2>
__global__ void k_snapshot_batch(void* const* __restrict__ works, void* const* __restrict__ states, uint32_t Ca,
                                 uint32_t Cb, const int* d_k) {
  const uint32_t m = blockIdx.z;
  transpose_tile(reinterpret_cast<const C2*>(works[m]), reinterpret_cast<C2*>(states[m]) + (uint64_t)*d_k * Ca * Cb,
                 Cb, Ca);
}

template <typename C2>
__global__ void k_load_batch(void* const* __restrict__ works, void* const* __restrict__ states, uint32_t Ca,
                             uint32_t Cb, uint32_t block) {
  const uint32_t m = blockIdx.z;
  transpose_tile(reinterpret_cast<const C2*>(states[m]) + (uint64_t)block * Ca * Cb,
                 reinterpret_cast<C2*>(works[m]), Ca, Cb);
}

// Continue the graph's while loop while the next power k + 1 is below `last`.
__global__ void k_continue_while(const int* d_k, int last, cudaGraphConditionalHandle h) {
  cudaGraphSetConditional(h, *d_k + 1 < last ? 1u : 0u);
}

static dim3 transpose_grid(uint32_t R, uint32_t C, uint32_t members) {
  return dim3((C + 31) / 32, (R + 31) / 32, members);
}

cudaError_t launch_snapshot(const void* work, void* state, uint32_t Ca, uint32_t Cb, const int* d_k, int dtype,
                            cudaStream_t s) {
  const dim3 g = transpose_grid(Cb, Ca, 1), b(32, 8);
  if (dtype == QPE_C128)
    k_snapshot<double2><<<g, b, 0, s>>>((const double2*)work, (double2*)state, Ca, Cb, d_k);
  else
    k_snapshot<float2><<<g, b, 0, s>>>((const float2*)work, (float2*)state, Ca, Cb, d_k);
  return cudaGetLastError();
}

cudaError_t launch_load(void* work, const void* state, uint32_t Ca, uint32_t Cb, uint32_t block, int dtype,
                        cudaStream_t s) {
  const dim3 g = transpose_grid(Ca, Cb, 1), b(32, 8);
  if (dtype == QPE_C128)
    k_load<double2><<<g, b, 0, s>>>((double2*)work, (const double2*)state, Ca, Cb, block);
  else
    k_load<float2><<<g, b, 0, s>>>((float2*)work, (const float2*)state, Ca, Cb, block);
  return cudaGetLastError();
}

cudaError_t launch_snapshot_batch(void* const* works, void* const* states, uint32_t Ca, uint32_t Cb, const int* d_k,
                                  uint32_t nmem, int dtype, cudaStream_t s) {
  const dim3 g = transpose_grid(Cb, Ca, nmem), b(32, 8);
  if (dtype == QPE_C128)
    k_snapshot_batch<double2><<<g, b, 0, s>>>(works, states, Ca, Cb, d_k);
  else
    k_snapshot_batch<float2><<<g, b, 0, s>>>(works, states, Ca, Cb, d_k);
  return cudaGetLastError();
}

cudaError_t launch_load_batch(void* const* works, void* const* states, uint32_t Ca, uint32_t Cb, uint32_t block,
                              uint32_t nmem, int dtype, cudaStream_t s) {
  const dim3 g = transpose_grid(Ca, Cb, nmem), b(32, 8);
  if (dtype == QPE_C128)
    k_load_batch<double2><<<g, b, 0, s>>>(works, states, Ca, Cb, block);
  else
    k_load_batch<float2><<<g, b, 0, s>>>(works, states, Ca, Cb, block);
  return cudaGetLastError();
}

cudaError_t launch_continue_while(const int* d_k, int last, cudaGraphConditionalHandle h, cudaStream_t s) {
  k_continue_while<<<1, 1, 0, s>>>(d_k, last, h);
  return cudaGetLastError();
}

cudaError_t launch_advance(int* d_k, cudaStream_t s) {
  k_advance<<<1, 1, 0, s>>>(d_k);
  return cudaGetLastError();
}

}  // namespace qpe
