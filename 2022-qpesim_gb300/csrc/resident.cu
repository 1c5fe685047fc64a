// resident.cu - the evolution with the working block resident in shared memory.
//
// One launch runs every controlled power of one or more instances. An instance
// is owned by one CTA (K = 1) or by a thread-block cluster of K CTAs whose
// shared memories together hold the Ca x Cb block, split by rows: CTA r of the
// cluster owns rows [r * Rk, (r + 1) * Rk). For every pass of a power the
// cluster's warps take the pass's tiles (program.h):
//   K = 1: tiles are processed in place in shared memory;
//   K > 1: row tiles are local to the CTA that owns the rows; column and
//          column-pair tiles are gathered from the cluster's shared memories
//          (distributed shared memory) into a warp-private stage, processed,
//          and scattered back.
// Column and column-pair tiles go round-robin over the cluster's CTAs (tile t to
// CTA t % K), so that a pass with fewer tiles than warps still spreads its FP64
// work over every SM of the cluster. A barrier (__syncthreads for K = 1, the
// cluster barrier otherwise) closes every pass. After a power each CTA copies its rows to block k of the register
// in global memory (the copy of cpp/time_evolution_over_terms.hpp:130-132, taken
// after the power), so block k = U^k block 0. In place (time_evolve_iqpe, :141-155)
// the CTA loads block `first`, applies last - first powers and writes block
// `first` after each. No thread waits on a flag: the
// only synchronisation is the hardware barrier, reached the same number of
// times by every CTA of the cluster.
#include <cooperative_groups.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include "kernels.h"
#include "group_ops.cuh"
#include "tile_ops.cuh"

namespace cg = cooperative_groups;

namespace qpe {

template <typename C2>
__device__ __forceinline__ C2* cta_ptr(C2* local, uint32_t rank, uint32_t K) {
  if (K == 1) return local;
  return cg::this_cluster().map_shared_rank(local, rank);
}

// Copies elements i = lane, lane + 32, ... < n for which ok(i) holds from
// *src(i) to *dst(i), U loads in flight per lane before their stores, so that
// distributed-shared-memory latency is paid once per U elements.
template <typename V, int U, class Ok, class Src, class Dst>
__device__ __forceinline__ void warp_copy(uint32_t n, uint32_t lane, Ok ok, Src src, Dst dst) {
  for (uint32_t base = lane; base < n; base += 32 * U) {
    V v[U];
#pragma unroll
    for (int u = 0; u < U; ++u) {
      const uint32_t i = base + 32 * u;
      if (i < n && ok(i)) v[u] = *src(i);
    }
#pragma unroll
    for (int u = 0; u < U; ++u) {
      const uint32_t i = base + 32 * u;
      if (i < n && ok(i)) *dst(i) = v[u];
    }
  }
}

// warp_copy for a group of gthreads threads (thread gt): elements gt, gt +
// gthreads, ...
template <typename V, int U, class Ok, class Src, class Dst>
__device__ __forceinline__ void group_copy(uint32_t n, uint32_t gt, uint32_t gthreads, Ok ok, Src src, Dst dst) {
  for (uint32_t base = gt; base < n; base += gthreads * U) {
    V v[U];
#pragma unroll
    for (int u = 0; u < U; ++u) {
      const uint32_t i = base + gthreads * u;
      if (i < n && ok(i)) v[u] = *src(i);
    }
#pragma unroll
    for (int u = 0; u < U; ++u) {
      const uint32_t i = base + gthreads * u;
      if (i < n && ok(i)) *dst(i) = v[u];
    }
  }
}

size_t resident_meta_bytes(uint32_t nops, uint32_t pool_words, uint32_t npasses, uint32_t Ca, uint32_t Cb) {
  return (size_t)nops * sizeof(DevOp) + (size_t)((pool_words + 3u) & ~3u) * 4 + (size_t)npasses * sizeof(Pass) +
         (size_t)(Ca + Cb) * 4;
}

// Stages the program's metadata in shared memory at `meta` (16-byte aligned), in
// the order resident_meta_bytes counts it: term descriptors, index pool, passes,
// alpha and beta line strings; the pointers are redirected to the copies. Every
// thread of the CTA takes part; the caller's next barrier publishes the copies.
__device__ __forceinline__ void stage_program(const ResidentInstance& I, unsigned char* meta, const DevOp*& ops,
                                              const uint32_t*& pool, const Pass*& passes, const uint32_t*& strA,
                                              const uint32_t*& strB) {
  const uint32_t Ca = I.Ca, Cb = I.Cb;
  DevOp* ops_s = reinterpret_cast<DevOp*>(meta);
  uint32_t* pool_s = reinterpret_cast<uint32_t*>(meta + (size_t)I.nops * sizeof(DevOp));
  Pass* passes_s = reinterpret_cast<Pass*>(pool_s + ((I.pool_words + 3u) & ~3u));
  uint32_t* strA_s = reinterpret_cast<uint32_t*>(passes_s + I.npasses);
  uint32_t* strB_s = strA_s + Ca;
  const uint4* osrc = reinterpret_cast<const uint4*>(I.ops);
  for (uint32_t i = threadIdx.x; i < I.nops * 2; i += blockDim.x) reinterpret_cast<uint4*>(ops_s)[i] = osrc[i];
  for (uint32_t i = threadIdx.x; i < I.pool_words; i += blockDim.x) pool_s[i] = I.pool[i];
  const uint32_t* psrc = reinterpret_cast<const uint32_t*>(I.passes);
  for (uint32_t i = threadIdx.x; i < I.npasses * (uint32_t)(sizeof(Pass) / 4); i += blockDim.x)
    reinterpret_cast<uint32_t*>(passes_s)[i] = psrc[i];
  for (uint32_t i = threadIdx.x; i < Ca; i += blockDim.x) strA_s[i] = I.strA[i];
  for (uint32_t i = threadIdx.x; i < Cb; i += blockDim.x) strB_s[i] = I.strB[i];
  ops = ops_s;
  pool = pool_s;
  passes = passes_s;
  strA = strA_s;
  strB = strB_s;
}

constexpr uint32_t kGroupWarps = 4;

// MS: the program's metadata (term descriptors, index pool, passes, line strings)
// is copied into every CTA's shared memory at the start, so that the term loop
// reads it at shared-memory latency instead of through L1 / L2.
// MG: column-pair (MIX) passes are processed by groups of kGroupWarps warps with
// every update split over a quad of lanes (group_ops.cuh), as in
// k_resident_group; group g stages its tile in the stages of its warps 4g ..
// 4g + 3 (stage_elems is per warp). Row and column passes, whose many short
// terms favour single warps, stay as below.
template <typename R, class A, bool MS, bool MG>
__global__ void __launch_bounds__(512) k_resident(const ResidentInstance* __restrict__ insts, uint32_t stage_elems) {
  using C2 = typename Cx<R>::T;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  // one element per four-warp group for the lanes of group_mix_ops without a pair
  __shared__ C2 scratch_s[16 / kGroupWarps];
  cg::cluster_group cl = cg::this_cluster();
  const uint32_t K = cl.num_blocks();
  const uint32_t rank = cl.block_rank();
  const ResidentInstance I = insts[blockIdx.x / K];
  const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5, wpc = blockDim.x >> 5;
  const uint32_t Ca = I.Ca, Cb = I.Cb, Rk = I.rows_per_cta;
  const uint32_t row0 = min(rank * Rk, Ca), row1 = min(row0 + Rk, Ca);
  C2* blk = reinterpret_cast<C2*>(smem_raw);
  C2* stage = blk + (size_t)Rk * Cb + (size_t)warp * stage_elems;
  C2* __restrict__ gstate = reinterpret_cast<C2*>(I.state);
  const uint64_t ld = (uint64_t)Ca * Cb;
  const uint32_t nown = (row1 - row0) * Cb;

  auto barrier = [&]() {
    if (K == 1) __syncthreads();
    else cl.sync();
  };
  // Generic pointer to element (a, b) of the cluster-distributed block.
  auto at = [&](uint32_t a, uint32_t b) -> C2* {
    const uint32_t r = a / Rk;
    return cta_ptr(blk, r, K) + (size_t)(a - r * Rk) * Cb + b;
  };

  const DevOp* ops = I.ops;
  const uint32_t* pool = I.pool;
  const Pass* passes = I.passes;
  const uint32_t* strA = I.strA;
  const uint32_t* strB = I.strB;
  if constexpr (MS) {
    const size_t head = ((size_t)Rk * Cb + (size_t)wpc * stage_elems) * sizeof(C2);
    stage_program(I, smem_raw + ((head + 15) & ~(size_t)15), ops, pool, passes, strA, strB);
  }
  constexpr bool G = !MS;
  // distributed-shared-memory loads in flight per lane in the tile gathers
  // (fewer for complex128, whose 16-byte elements cost registers)
  constexpr int kGatherDepth = sizeof(R) == 8 ? 2 : 4;

  // Block first - 1 (block first when evolving in place) into shared memory.
  {
    const C2* src = gstate + (uint64_t)(I.in_place ? I.first : I.first - 1) * ld + (uint64_t)row0 * Cb;
    for (uint32_t i = threadIdx.x; i < nown; i += blockDim.x) blk[i] = src[i];
  }
  barrier();

  const uint32_t nsweeps = I.steps * I.order;
  for (uint32_t k = I.first; k < I.last; ++k) {
    for (uint32_t sw = 0; sw < nsweeps; ++sw) {
    // Second-order steps alternate a forward and a backward sweep; the backward
    // sweep runs the passes, and each pass's terms, in reverse order.
    const bool rev = I.order == 2 && (sw & 1);
    for (uint32_t pj = 0; pj < I.npasses; ++pj) {
      const uint32_t pi = rev ? I.npasses - 1 - pj : pj;
      const Pass P = passes[pi];
      if (P.type == PASS_ROW) {
        // Rows owned by this CTA, Wr rows per warp tile, in place.
        const uint32_t W = I.Wr, logW = __ffs(W) - 1, w = lane & (W - 1);
        const uint32_t jl = lane >> logW, jstep = 32 >> logW;
        const uint32_t ntiles = (row1 - row0 + W - 1) >> logW;
        for (uint32_t tile = warp; tile < ntiles; tile += wpc) {
          const uint32_t r = row0 + (tile << logW) + w;
          const bool active = r < row1;
          const uint32_t lstr = active ? ldm<G>(strA + r) : 0u;
          C2* line = blk + (size_t)(active ? r - row0 : 0) * Cb;
          run_line_ops<R, A, G>(ops, I.coef, pool, P.op0, P.op1, rev, Cb, jl, jstep, active, lstr,
                             [&](uint32_t e) -> C2& { return line[e]; });
        }
      } else if (P.type == PASS_COL) {
        const uint32_t W = I.Wc, logW = __ffs(W) - 1, w = lane & (W - 1);
        const uint32_t jl = lane >> logW, jstep = 32 >> logW;
        const uint32_t ntiles = (Cb + W - 1) >> logW;
        const uint32_t gw = warp * K + rank, nw = K * wpc;  // tile t on CTA t % K
        for (uint32_t tile = gw; tile < ntiles; tile += nw) {
          const uint32_t b0 = tile << logW, c = b0 + w;
          const bool active = c < Cb;
          const uint32_t lstr = active ? ldm<G>(strB + c) : 0u;
          if (K == 1) {
            C2* col = blk + (active ? c : 0);
            run_line_ops<R, A, G>(ops, I.coef, pool, P.op0, P.op1, rev, Ca, jl, jstep, active, lstr,
                               [&](uint32_t e) -> C2& { return col[(size_t)e * Cb]; });
          } else {
            const uint32_t nl = min(W, Cb - b0);
            auto ok = [&](uint32_t i) { return (i & (W - 1)) < nl; };
            auto remote = [&](uint32_t i) { return at(i >> logW, b0 + (i & (W - 1))); };
            auto local = [&](uint32_t i) { return stage + i; };
            warp_copy<C2, kGatherDepth>(Ca << logW, lane, ok, remote, local);
            __syncwarp();
            run_line_ops<R, A, G>(ops, I.coef, pool, P.op0, P.op1, rev, Ca, jl, jstep, active, lstr,
                               [&](uint32_t e) -> C2& { return stage[(e << logW) + w]; });
            warp_copy<C2, kGatherDepth>(Ca << logW, lane, ok, local, remote);
            __syncwarp();
          }
        }
      } else if constexpr (MG) {  // PASS_MIX by four-warp groups: Wm column pairs per group tile
        const uint32_t gthreads = 32 * kGroupWarps, ngrp = wpc / kGroupWarps;
        const uint32_t grp = warp / kGroupWarps, gt = threadIdx.x - grp * gthreads;
        C2* gstage = blk + (size_t)Rk * Cb + (size_t)grp * kGroupWarps * stage_elems;
        auto gbar = [&]() { asm volatile("bar.sync %0, %1;" ::"r"(1 + grp), "r"(gthreads) : "memory"); };
        const uint32_t W = I.Wm, logW = __ffs(W) - 1;
        const uint32_t ntiles = (P.mixcount + W - 1) >> logW;
        const uint2* __restrict__ mt = reinterpret_cast<const uint2*>(pool + P.mixtab);
        for (uint32_t tile = grp * K + rank; tile < ntiles; tile += K * ngrp) {
          const uint32_t t0 = tile << logW, nv = min(W, P.mixcount - t0);
          auto pair_of = [&](uint32_t w) { return ldm<G>(mt + t0 + w); };
          auto parb = [&](uint32_t w) { return pair_of(w).x >> 31; };
          if (K == 1) {
            auto left = [&](uint32_t w, uint32_t a) -> C2& {
              return blk[(size_t)a * Cb + (pair_of(w).x & 0x7fffffffu)];
            };
            auto right = [&](uint32_t w, uint32_t a) -> C2& { return blk[(size_t)a * Cb + pair_of(w).y]; };
            group_mix_ops<R, A, G>(ops, I.coef, pool, P.op0, P.op1, rev, logW, nv, gt, gthreads, left, right, parb,
                                   gbar, scratch_s + grp);
          } else {
            // element i: row i >> (logW + 1), column pair (i >> 1) & (W - 1), side i & 1; with
            // gthreads a multiple of 2W a thread's column is the same for all its elements
            const uint32_t mysel = gt & (2 * W - 1);
            const uint2 myq = ((mysel >> 1) < nv) ? pair_of(mysel >> 1) : make_uint2(0u, 0u);
            const uint32_t mycol = (mysel & 1) ? myq.y : (myq.x & 0x7fffffffu);
            auto ok = [&](uint32_t) { return (mysel >> 1) < nv; };
            auto remote = [&](uint32_t i) { return at(i >> (logW + 1), mycol); };
            auto local = [&](uint32_t i) { return gstage + i; };
            const uint32_t n2 = Ca << (logW + 1);
            group_copy<C2, kGatherDepth>(n2, gt, gthreads, ok, remote, local);
            gbar();
            auto left = [&](uint32_t w, uint32_t a) -> C2& { return gstage[(a << (logW + 1)) + 2 * w]; };
            auto right = [&](uint32_t w, uint32_t a) -> C2& { return gstage[(a << (logW + 1)) + 2 * w + 1]; };
            group_mix_ops<R, A, G>(ops, I.coef, pool, P.op0, P.op1, rev, logW, nv, gt, gthreads, left, right, parb,
                                   gbar, scratch_s + grp);
            group_copy<C2, kGatherDepth>(n2, gt, gthreads, ok, local, remote);
            gbar();
          }
        }
      } else {  // PASS_MIX: Wm column pairs per tile
        const uint32_t W = I.Wm, logW = __ffs(W) - 1, w = lane & (W - 1);
        const uint32_t jl = lane >> logW, jstep = 32 >> logW;
        const uint32_t ntiles = (P.mixcount + W - 1) >> logW;
        const uint32_t gw = warp * K + rank, nw = K * wpc;  // tile t on CTA t % K
        const uint2* __restrict__ mt = reinterpret_cast<const uint2*>(pool + P.mixtab);
        for (uint32_t tile = gw; tile < ntiles; tile += nw) {
          const uint32_t t0 = tile << logW, t = t0 + w;
          const bool active = t < P.mixcount;
          const uint2 bp = active ? ldm<G>(mt + t) : make_uint2(0u, 0u);
          const uint32_t b01 = bp.x & 0x7fffffffu, b10 = bp.y, parb = bp.x >> 31;
          if (K == 1) {
            run_mix_ops<R, A, G>(ops, I.coef, pool, P.op0, P.op1, rev, jl, jstep, active, parb,
                              [&](uint32_t a) -> C2& { return blk[(size_t)a * Cb + b01]; },
                              [&](uint32_t a) -> C2& { return blk[(size_t)a * Cb + b10]; });
          } else {
            const uint32_t nl = min(W, P.mixcount - t0);
            const uint32_t n2 = Ca << (logW + 1);
            // lane's column of element i: column-pair (i >> 1) & (W - 1), side i & 1;
            // with 32 a multiple of 2W it is the same for every i of the lane.
            const uint32_t mysel = lane & (2 * W - 1);
            const uint2 myq = ((mysel >> 1) < nl) ? ldm<G>(mt + t0 + (mysel >> 1)) : make_uint2(0u, 0u);
            const uint32_t mycol = (mysel & 1) ? myq.y : (myq.x & 0x7fffffffu);
            auto ok = [&](uint32_t) { return (mysel >> 1) < nl; };
            auto remote = [&](uint32_t i) { return at(i >> (logW + 1), mycol); };
            auto local = [&](uint32_t i) { return stage + i; };
            warp_copy<C2, kGatherDepth>(n2, lane, ok, remote, local);
            __syncwarp();
            run_mix_ops<R, A, G>(ops, I.coef, pool, P.op0, P.op1, rev, jl, jstep, active, parb,
                              [&](uint32_t a) -> C2& { return stage[(a << (logW + 1)) + 2 * w]; },
                              [&](uint32_t a) -> C2& { return stage[(a << (logW + 1)) + 2 * w + 1]; });
            warp_copy<C2, kGatherDepth>(n2, lane, ok, local, remote);
            __syncwarp();
          }
        }
      }
      barrier();
    }
    }
    // Snapshot of this CTA's rows into block k (block first when in place).
    C2* dst = gstate + (uint64_t)(I.in_place ? I.first : k) * ld + (uint64_t)row0 * Cb;
    for (uint32_t i = threadIdx.x; i < nown; i += blockDim.x) dst[i] = blk[i];
    barrier();
  }
}

// The same evolution with tiles processed by groups of four warps (one per SM
// sub-partition) and every update split over a quad of lanes (group_ops.cuh):
// a term's FP64 work is spread over the four FP64 units of the SM instead of
// one. Tiles (rows, columns or column pairs) go to the cluster's groups
// round-robin; stage_elems is per group.

template <typename R, class A, bool MS>
__global__ void __launch_bounds__(512) k_resident_group(const ResidentInstance* __restrict__ insts,
                                                        uint32_t stage_elems) {
  using C2 = typename Cx<R>::T;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ C2 scratch_s[16 / kGroupWarps];  // as in k_resident
  cg::cluster_group cl = cg::this_cluster();
  const uint32_t K = cl.num_blocks();
  const uint32_t rank = cl.block_rank();
  const ResidentInstance I = insts[blockIdx.x / K];
  const uint32_t wpc = blockDim.x >> 5;
  const uint32_t gthreads = 32 * kGroupWarps, ngrp = wpc / kGroupWarps;
  const uint32_t grp = threadIdx.x / gthreads, gt = threadIdx.x - grp * gthreads;
  const uint32_t Ca = I.Ca, Cb = I.Cb, Rk = I.rows_per_cta;
  const uint32_t row0 = min(rank * Rk, Ca), row1 = min(row0 + Rk, Ca);
  C2* blk = reinterpret_cast<C2*>(smem_raw);
  C2* stage = blk + (size_t)Rk * Cb + (size_t)grp * stage_elems;
  C2* __restrict__ gstate = reinterpret_cast<C2*>(I.state);
  const uint64_t ld = (uint64_t)Ca * Cb;
  const uint32_t nown = (row1 - row0) * Cb;

  auto barrier = [&]() {
    if (K == 1) __syncthreads();
    else cl.sync();
  };
  auto gbar = [&]() { asm volatile("bar.sync %0, %1;" ::"r"(1 + grp), "r"(gthreads) : "memory"); };
  auto at = [&](uint32_t a, uint32_t b) -> C2* {
    const uint32_t r = a / Rk;
    return cta_ptr(blk, r, K) + (size_t)(a - r * Rk) * Cb + b;
  };

  const DevOp* ops = I.ops;
  const uint32_t* pool = I.pool;
  const Pass* passes = I.passes;
  const uint32_t* strA = I.strA;
  const uint32_t* strB = I.strB;
  if constexpr (MS) {
    const size_t head = ((size_t)Rk * Cb + (size_t)ngrp * stage_elems) * sizeof(C2);
    stage_program(I, smem_raw + ((head + 15) & ~(size_t)15), ops, pool, passes, strA, strB);
  }
  constexpr bool G = !MS;
  constexpr int kDepth = sizeof(R) == 8 ? 2 : 4;
  auto no_parity = [](uint32_t) { return 0u; };

  {
    const C2* src = gstate + (uint64_t)(I.in_place ? I.first : I.first - 1) * ld + (uint64_t)row0 * Cb;
    for (uint32_t i = threadIdx.x; i < nown; i += blockDim.x) blk[i] = src[i];
  }
  barrier();

  const uint32_t nsweeps = I.steps * I.order;
  for (uint32_t k = I.first; k < I.last; ++k) {
    for (uint32_t sw = 0; sw < nsweeps; ++sw) {
      const bool rev = I.order == 2 && (sw & 1);
      for (uint32_t pj = 0; pj < I.npasses; ++pj) {
        const uint32_t pi = rev ? I.npasses - 1 - pj : pj;
        const Pass P = passes[pi];
        if (P.type == PASS_ROW) {
          // this CTA's rows, Wr per group tile, in place
          const uint32_t W = I.Wr, logW = __ffs(W) - 1;
          const uint32_t ntiles = (row1 - row0 + W - 1) >> logW;
          for (uint32_t tile = grp; tile < ntiles; tile += ngrp) {
            const uint32_t r0 = row0 + (tile << logW), nv = min(W, row1 - r0);
            auto line = [&](uint32_t w, uint32_t e) -> C2& { return blk[(size_t)(r0 - row0 + w) * Cb + e]; };
            group_ops<R, A, G>(ops, I.coef, pool, P.op0, P.op1, rev, Cb, logW, nv, false, gt, gthreads, line, line,
                               [&](uint32_t w) { return ldm<G>(strA + r0 + w); }, no_parity, gbar);
          }
        } else if (P.type == PASS_COL) {
          const uint32_t W = I.Wc, logW = __ffs(W) - 1;
          const uint32_t ntiles = (Cb + W - 1) >> logW;
          for (uint32_t tile = grp * K + rank; tile < ntiles; tile += K * ngrp) {
            const uint32_t b0 = tile << logW, nv = min(W, Cb - b0);
            auto lstr = [&](uint32_t w) { return ldm<G>(strB + b0 + w); };
            if (K == 1) {
              auto line = [&](uint32_t w, uint32_t e) -> C2& { return blk[(size_t)e * Cb + b0 + w]; };
              group_ops<R, A, G>(ops, I.coef, pool, P.op0, P.op1, rev, Ca, logW, nv, false, gt, gthreads, line, line,
                                 lstr, no_parity, gbar);
            } else {
              auto ok = [&](uint32_t i) { return (i & (W - 1)) < nv; };
              auto remote = [&](uint32_t i) { return at(i >> logW, b0 + (i & (W - 1))); };
              auto local = [&](uint32_t i) { return stage + i; };
              group_copy<C2, kDepth>(Ca << logW, gt, gthreads, ok, remote, local);
              gbar();
              auto line = [&](uint32_t w, uint32_t e) -> C2& { return stage[(e << logW) + w]; };
              group_ops<R, A, G>(ops, I.coef, pool, P.op0, P.op1, rev, Ca, logW, nv, false, gt, gthreads, line, line,
                                 lstr, no_parity, gbar);
              group_copy<C2, kDepth>(Ca << logW, gt, gthreads, ok, local, remote);
              gbar();
            }
          }
        } else {  // PASS_MIX: Wm column pairs per group tile
          const uint32_t W = I.Wm, logW = __ffs(W) - 1;
          const uint32_t ntiles = (P.mixcount + W - 1) >> logW;
          const uint2* __restrict__ mt = reinterpret_cast<const uint2*>(pool + P.mixtab);
          for (uint32_t tile = grp * K + rank; tile < ntiles; tile += K * ngrp) {
            const uint32_t t0 = tile << logW, nv = min(W, P.mixcount - t0);
            auto pair_of = [&](uint32_t w) { return ldm<G>(mt + t0 + w); };
            auto parb = [&](uint32_t w) { return pair_of(w).x >> 31; };
            if (K == 1) {
              auto left = [&](uint32_t w, uint32_t a) -> C2& {
                return blk[(size_t)a * Cb + (pair_of(w).x & 0x7fffffffu)];
              };
              auto right = [&](uint32_t w, uint32_t a) -> C2& { return blk[(size_t)a * Cb + pair_of(w).y]; };
              group_mix_ops<R, A, G>(ops, I.coef, pool, P.op0, P.op1, rev, logW, nv, gt, gthreads, left, right, parb,
                                     gbar, scratch_s + grp);
            } else {
              // element i: row i >> (logW + 1), column pair (i >> 1) & (W - 1), side i & 1; with
              // gthreads a multiple of 2W a thread's column is the same for all its elements
              const uint32_t mysel = gt & (2 * W - 1);
              const uint2 myq = ((mysel >> 1) < nv) ? pair_of(mysel >> 1) : make_uint2(0u, 0u);
              const uint32_t mycol = (mysel & 1) ? myq.y : (myq.x & 0x7fffffffu);
              auto ok = [&](uint32_t) { return (mysel >> 1) < nv; };
              auto remote = [&](uint32_t i) { return at(i >> (logW + 1), mycol); };
              auto local = [&](uint32_t i) { return stage + i; };
              const uint32_t n2 = Ca << (logW + 1);
              group_copy<C2, kDepth>(n2, gt, gthreads, ok, remote, local);
              gbar();
              auto left = [&](uint32_t w, uint32_t a) -> C2& { return stage[(a << (logW + 1)) + 2 * w]; };
              auto right = [&](uint32_t w, uint32_t a) -> C2& { return stage[(a << (logW + 1)) + 2 * w + 1]; };
              group_mix_ops<R, A, G>(ops, I.coef, pool, P.op0, P.op1, rev, logW, nv, gt, gthreads, left, right, parb,
                                     gbar, scratch_s + grp);
              group_copy<C2, kDepth>(n2, gt, gthreads, ok, local, remote);
              gbar();
            }
          }
        }
        barrier();
      }
    }
    C2* dst = gstate + (uint64_t)(I.in_place ? I.first : k) * ld + (uint64_t)row0 * Cb;
    for (uint32_t i = threadIdx.x; i < nown; i += blockDim.x) dst[i] = blk[i];
    barrier();
  }
}

// Every tile processed by a group of three warps with the lean runners
// (group_ops.cuh): one column, one row or one column pair per group tile, pair
// updates split over quads and diagonal updates over lane pairs, the partner
// operand by shuffle. Three-warp groups give a cluster of 16 CTAs of 15 warps
// 80 groups, more than the 70 columns of an n = 16 block, so that the long
// first column pass runs one column per group; a term of up to 24 pairs or 48
// diagonal entries is one update per lane. Tiles go round-robin over the
// cluster's groups; rows are processed by the CTA that owns them.
constexpr uint32_t kLeanWarps = 3;

template <typename R, class A, bool MS, bool REP>
__global__ void __launch_bounds__(480) k_resident_lean(const ResidentInstance* __restrict__ insts,
                                                       uint32_t stage_elems) {
  using C2 = typename Cx<R>::T;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ C2 scratch_s[16 / kLeanWarps];  // per group: target of the lanes without an update
  cg::cluster_group cl = cg::this_cluster();
  const uint32_t K = cl.num_blocks();
  const uint32_t rank = cl.block_rank();
  // Replica clusters (REP: the same number for every instance of a launch) and
  // this cluster's replica, recomputed where needed rather than kept in registers.
  auto nrep_f = [&]() { return REP && K > 1 ? max(__ldg(&insts[0].replicas), 1u) : 1u; };
  auto rep_f = [&]() { return (blockIdx.x / K) % nrep_f(); };
  const ResidentInstance I = insts[blockIdx.x / (K * nrep_f())];
  const uint32_t wpc = blockDim.x >> 5;
  const uint32_t gthreads = 32 * kLeanWarps, ngrp = wpc / kLeanWarps;
  const uint32_t grp = threadIdx.x / gthreads, gt = threadIdx.x - grp * gthreads;
  const uint32_t Ca = I.Ca, Cb = I.Cb, Rk = I.rows_per_cta;
  const uint32_t row0 = min(rank * Rk, Ca), row1 = min(row0 + Rk, Ca);
  C2* blk = reinterpret_cast<C2*>(smem_raw);
  C2* stage = blk + (size_t)Rk * Cb + (size_t)grp * stage_elems;
  C2* __restrict__ gstate = reinterpret_cast<C2*>(I.state);
  C2* scratch = scratch_s + grp;
  const uint64_t ld = (uint64_t)Ca * Cb;
  const uint32_t nown = (row1 - row0) * Cb;

  auto barrier = [&]() {
    if (K == 1) __syncthreads();
    else cl.sync();
  };
  auto gbar = [&]() { asm volatile("bar.sync %0, %1;" ::"r"(1 + grp), "r"(gthreads) : "memory"); };
  // Row a of the cluster-distributed block starts at rowp[a] (a generic pointer
  // into the owning CTA's shared memory), so that a gather or scatter element
  // costs one shared load instead of a division and an address mapping.
  const size_t head = ((size_t)Rk * Cb + (size_t)ngrp * stage_elems) * sizeof(C2);
  C2** rowp = reinterpret_cast<C2**>(smem_raw + ((head + 15) & ~(size_t)15));
  for (uint32_t a = threadIdx.x; a < Ca; a += blockDim.x) {
    const uint32_t r = a / Rk;
    rowp[a] = cta_ptr(blk, r, K) + (size_t)(a - r * Rk) * Cb;
  }
  auto at = [&](uint32_t a, uint32_t b) -> C2* { return rowp[a] + b; };
  // Column-pair update units (mix_units.h): this warp's program slot follows the
  // row-pointer table; the slot holds the program of window wp_pass (or its copy
  // on the way, cp.async).
  const uint32_t wpw = (K > 1 && I.mix_words) ? I.mix_wp_words : 0u;
  const uint32_t warp = threadIdx.x >> 5, lane = threadIdx.x & 31u;
  unsigned char* const wp_base =
      smem_raw + ((head + 15) & ~(size_t)15) + (((size_t)Ca * sizeof(C2*) + 15) & ~(size_t)15);
  uint32_t* const wp_s = reinterpret_cast<uint32_t*>(wp_base) + (size_t)warp * wpw;
  uint32_t wp_pass = kMixNoSchedule;

  const DevOp* ops = I.ops;
  const uint32_t* pool = I.pool;
  const Pass* passes = I.passes;
  const uint32_t* strA = I.strA;
  const uint32_t* strB = I.strB;
  if constexpr (MS)
    stage_program(I, wp_base + (size_t)wpc * wpw * 4, ops, pool, passes, strA, strB);
  constexpr bool G = !MS;
  constexpr int kDepth = sizeof(R) == 8 ? 2 : 4;
  const bool in_group = grp < ngrp;  // threads past the last whole group only join the CTA barriers

  {
    const C2* src = gstate + (uint64_t)(I.in_place ? I.first : I.first - 1) * ld + (uint64_t)row0 * Cb;
    for (uint32_t i = threadIdx.x; i < nown; i += blockDim.x) blk[i] = src[i];
  }
  barrier();

  // Replica exchange after a row or column pass that the replicas split: this
  // CTA publishes the amplitudes of its rows that its replica computed (element
  // (a, b) belongs to replica b % nrep after a column pass, (a - row0) % nrep
  // after a row pass) into buffer g % 2 for exchange g, raises its exchange
  // count to g, waits (bounded) until the same CTA of every other replica has
  // done so, and takes their amplitudes. Two buffers suffice: a replica writes
  // exchange g + 2 only after the others' counts reached g + 1, which each
  // raises after its reads of exchange g. Once a wait runs out
  // (kResidentErrExchange ORed into *err) the CTA stops waiting. The exchange
  // count and that state live in shared memory.
  __shared__ uint32_t xstate;  // exchanges done << 1 | a wait ran out
  if (threadIdx.x == 0) xstate = 0;
  auto exchange = [&](bool col) {
    const uint32_t nrep = nrep_f(), rep = rep_f();
    const uint32_t xs = xstate, xgen = (xs >> 1) + 1;
    C2* const xb = reinterpret_cast<C2*>(I.xbuf) + (size_t)(xgen & 1u) * ld + (size_t)row0 * Cb;
    auto owner = [&](uint32_t i) { return (col ? i % Cb : i / Cb) % nrep; };
    for (uint32_t i = threadIdx.x; i < nown; i += blockDim.x)
      if (owner(i) == rep) xb[i] = blk[i];
    __syncthreads();
    if (threadIdx.x == 0) {
      __threadfence();
      asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(I.xflag + rep * K + rank), "r"(xgen) : "memory");
    }
    bool late = false;
    if (threadIdx.x < nrep && threadIdx.x != rep && !(xs & 1u)) {
      const uint32_t* f = I.xflag + threadIdx.x * K + rank;
      for (uint32_t it = 0;; ++it) {
        uint32_t v;
        asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(f) : "memory");
        if (v >= xgen) break;
        if (it == (1u << 20)) {
          late = true;
          break;
        }
        __nanosleep(128);
      }
    }
    const bool failed = __syncthreads_or(late) || (xs & 1u);
    if (threadIdx.x == 0) {
      if (failed && !(xs & 1u)) atomicOr(I.err, kResidentErrExchange);  // the first wait of this CTA that ran out
      xstate = (xgen << 1) | (failed ? 1u : 0u);
    }
    for (uint32_t i = threadIdx.x; i < nown; i += blockDim.x)
      if (owner(i) != rep) blk[i] = __ldcg(xb + i);
  };

  const uint32_t nsweeps = I.steps * I.order;
  // per pass: kMixNoSchedule, or its window's block of warp programs (bits 0-19)
  // and the window's passes (bits 20-27)
  auto mix_slot = [&](uint32_t pi) { return wpw ? __ldg(I.mix_slot + pi) : kMixNoSchedule; };
  // Copies this warp's program of the window of pass pi (if it has one) into its
  // slot; every lane of the warp calls it. A copy still on its way is waited for
  // first.
  auto wp_fetch = [&](uint32_t pi) {
    const uint32_t m = mix_slot(pi);
    if (m == kMixNoSchedule || wp_pass == (m & 0xfffffu)) return;
    asm volatile("cp.async.wait_all;" ::: "memory");
    __syncwarp();
    const uint32_t* src = I.mix_words + (((size_t)(m & 0xfffffu) * K + rank) * wpc + warp) * wpw;
    for (uint32_t c = lane; c < wpw / 4; c += 32) {
      const uint32_t d = (uint32_t)__cvta_generic_to_shared(wp_s + 4 * c);
      asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(d), "l"(src + 4 * c) : "memory");
    }
    asm volatile("cp.async.commit_group;" ::: "memory");
    wp_pass = m & 0xfffffu;
  };
  auto pass_at = [&](uint32_t sw, uint32_t pj) { return (I.order == 2 && (sw & 1)) ? I.npasses - 1 - pj : pj; };
  for (uint32_t k = I.first; k < I.last; ++k) {
    for (uint32_t sw = 0; sw < nsweeps; ++sw) {
      const bool rev = I.order == 2 && (sw & 1);
      for (uint32_t pj = 0; pj < I.npasses; ++pj) {
        const uint32_t pi = rev ? I.npasses - 1 - pj : pj;
        const Pass P = passes[pi];
        const uint32_t m = P.type == PASS_MIX ? mix_slot(pi) : kMixNoSchedule;
        // a window of w passes is met at its first pass in either direction (the
        // passes are consecutive) and runs them all: the loop skips the rest
        const uint32_t span = m == kMixNoSchedule ? 1u : (m >> 20) & 0xffu;
        const uint32_t nj = pj + span;
        const uint32_t next_pi = nj < I.npasses ? pass_at(sw, nj) : pass_at(sw + 1 < nsweeps ? sw + 1 : 0, 0);
        if (!in_group) {
          // no tile
        } else if (m != kMixNoSchedule) {
          // this warp's share of the window's update units: gather its amplitudes
          // into the group's stage, one level per term (quad u of the warp does
          // update u of the level, split over its four lanes as in the tile
          // runner), scatter them back
          wp_fetch(pi);
          asm volatile("cp.async.wait_all;" ::: "memory");
          __syncwarp();
          const uint32_t hdr = wp_s[0], op0 = wp_s[1];
          const uint32_t tw = (hdr >> 7) & 3u;
          if (tw) {
            auto tsync = [&]() {
              if (tw == 1) __syncwarp();
              else asm volatile("bar.sync %0, %1;" ::"r"(1 + grp), "r"(32 * tw) : "memory");
            };
            C2* const gst = blk + (size_t)Rk * Cb + (size_t)grp * stage_elems;
            // up to two amplitudes per lane: entries lane and lane + 32
            const uint32_t nel = hdr & 127u, nlev = (hdr >> 9) & 0xffu;
            const uint32_t gw = lane < nel ? wp_s[kMixWpHeader + lane] : 0u;
            const uint32_t gw2 = lane + 32 < nel ? wp_s[kMixWpHeader + 32 + lane] : 0u;
            C2* const gp = at(gw & 2047u, (gw >> 11) & 2047u);
            C2* const sp = gst + (gw >> 22);
            C2* const gp2 = at(gw2 & 2047u, (gw2 >> 11) & 2047u);
            C2* const sp2 = gst + (gw2 >> 22);
            if (lane < nel) {
              const C2 v = *gp;
              if (lane + 32 < nel) *sp2 = *gp2;
              *sp = v;
            }
            tsync();
            const uint32_t q = lane & 3u, quad = lane >> 2;
            const bool side1 = q >= 2;
            const uint32_t comp1 = q & 1u, sflip = comp1 ^ 1u;
            R* const gr = reinterpret_cast<R*>(gst);
            // the next level's update word and coefficients are loaded a level ahead
            uint32_t lv_n = rev ? nlev - 1 : 0;
            uint32_t uw_n = wp_s[kMixWpHeader + kMixWarpAmps + 8 * lv_n + quad];
            uint4 b_n = ldm<G>(reinterpret_cast<const uint4*>(ops + op0 + lv_n) + 1);
            for (uint32_t i = 0; i < nlev; ++i) {
              const uint32_t uw = uw_n;
              const uint4 b = b_n;
              if (i + 1 < nlev) {
                lv_n = rev ? nlev - 2 - i : i + 1;
                uw_n = wp_s[kMixWpHeader + kMixWarpAmps + 8 * lv_n + quad];
                b_n = ldm<G>(reinterpret_cast<const uint4*>(ops + op0 + lv_n) + 1);
              }
              const R c = (R)__hiloint2double((int)b.y, (int)b.x), t = (R)__hiloint2double((int)b.w, (int)b.z);
              const bool v = (uw >> 21) & 1u;
              R* const dp = gr + 2 * (side1 ? ((uw >> 10) & 1023u) : (uw & 1023u)) + comp1;
              const R x1 = v ? *dp : (R)0;
              const R x2 = __shfl_xor_sync(0xffffffffu, x1, 3);
              if (v) *dp = A::add(A::mul(x1, c), A::mul(x2, (((uw >> 20) & 1u) ^ sflip) ? neg(t) : t));
              tsync();
            }
            if (lane < nel) *gp = *sp;
            if (lane + 32 < nel) *gp2 = *sp2;
          }
        } else if (K > 1 && I.line_slot && __ldg(I.line_slot + pi) != kMixNoSchedule) {
          // a row or column pass as per-line programs (mix_units.h): this warp's
          // share of its group's line, if it has one
          const uint32_t off =
              __ldg(I.line_offs + (((size_t)__ldg(I.line_slot + pi) * nrep_f() + rep_f()) * K + rank) * wpc + warp);
          if (off != kMixNoSchedule) {
            const uint32_t* const prog = I.line_words + off;
            const uint32_t hdr = __ldg(prog), nlev = __ldg(prog + 1);
            const uint32_t tw = (hdr >> 7) & 3u, nel = hdr & 127u;
            auto tsync = [&]() {
              if (tw == 1) __syncwarp();
              else asm volatile("bar.sync %0, %1;" ::"r"(1 + grp), "r"(32 * tw) : "memory");
            };
            C2* const gst = blk + (size_t)Rk * Cb + (size_t)grp * stage_elems;
            const uint32_t gw = lane < nel ? __ldg(prog + kMixWpHeader + lane) : 0u;
            const uint32_t gw2 = lane + 32 < nel ? __ldg(prog + kMixWpHeader + 32 + lane) : 0u;
            C2* const gp = at(gw & 2047u, (gw >> 11) & 2047u);
            C2* const sp = gst + (gw >> 22);
            C2* const gp2 = at(gw2 & 2047u, (gw2 >> 11) & 2047u);
            C2* const sp2 = gst + (gw2 >> 22);
            if (lane < nel) {
              const C2 v = *gp;
              if (lane + 32 < nel) *sp2 = *gp2;
              *sp = v;
            }
            tsync();
            // levels: op word (index in the pass | diagonal << 31) and this quad's
            // update word, streamed from global memory three levels ahead; the
            // coefficients one level ahead
            const uint32_t* const lw = prog + kMixWpHeader + kMixWarpAmps;
            const uint32_t q = lane & 3u, quad = lane >> 2;
            const bool side1 = q >= 2;
            const uint32_t comp1 = q & 1u, sflip = comp1 ^ 1u, half = (lane >> 1) & 1u, hh = lane & 1u;
            R* const gr = reinterpret_cast<R*>(gst);
            auto at_lv = [&](uint32_t i) { return lw + 9 * (size_t)(rev ? nlev - 1 - i : i); };
            uint32_t o0 = 0, u0 = 0, o1 = 0, u1 = 0, o2 = 0, u2 = 0;
            if (nlev > 0) { o0 = __ldg(at_lv(0)); u0 = __ldg(at_lv(0) + 1 + quad); }
            if (nlev > 1) { o1 = __ldg(at_lv(1)); u1 = __ldg(at_lv(1) + 1 + quad); }
            if (nlev > 2) { o2 = __ldg(at_lv(2)); u2 = __ldg(at_lv(2) + 1 + quad); }
            uint4 b_n = ldm<G>(reinterpret_cast<const uint4*>(ops + P.op0 + (o0 & 0xffffffu)) + 1);
            for (uint32_t i = 0; i < nlev; ++i) {
              const uint32_t opw = o0, uw = u0;
              const uint4 b = b_n;
              o0 = o1; u0 = u1; o1 = o2; u1 = u2;
              if (i + 3 < nlev) { o2 = __ldg(at_lv(i + 3)); u2 = __ldg(at_lv(i + 3) + 1 + quad); }
              if (i + 1 < nlev) b_n = ldm<G>(reinterpret_cast<const uint4*>(ops + P.op0 + (o0 & 0xffffffu)) + 1);
              const R c = (R)__hiloint2double((int)b.y, (int)b.x), t = (R)__hiloint2double((int)b.w, (int)b.z);
              if (opw >> 31) {
                // diagonal: lanes 4u, 4u + 1 take the word's first amplitude, 4u + 2, 4u + 3 its second;
                // lane h writes component h of v (c + i t)
                const bool v = (uw >> (20 + half)) & 1u;
                R* const dp = gr + 2 * ((uw >> (10 * half)) & 1023u) + hh;
                const R x1 = v ? *dp : (R)0;
                const R x2 = __shfl_xor_sync(0xffffffffu, x1, 1);
                if (v) *dp = A::add(A::mul(x1, c), A::mul(x2, hh ? t : neg(t)));
              } else {
                const bool v = (uw >> 21) & 1u;
                R* const dp = gr + 2 * (side1 ? ((uw >> 10) & 1023u) : (uw & 1023u)) + comp1;
                const R x1 = v ? *dp : (R)0;
                const R x2 = __shfl_xor_sync(0xffffffffu, x1, 3);
                if (v) *dp = A::add(A::mul(x1, c), A::mul(x2, (((uw >> 20) & 1u) ^ sflip) ? neg(t) : t));
              }
              tsync();
            }
            if (lane < nel) *gp = *sp;
            if (lane + 32 < nel) *gp2 = *sp2;
          }
        } else if (P.type == PASS_ROW) {
          // this CTA's rows of this replica, one per group tile, in place
          const uint32_t nrep = nrep_f();
          for (uint32_t r = row0 + rep_f() + nrep * grp; r < row1; r += nrep * ngrp) {
            C2* line = blk + (size_t)(r - row0) * Cb;
            group_line_ops<R, A, G>(ops, I.coef, pool, P.op0, P.op1, rev, Cb, ldm<G>(strA + r), gt, gthreads,
                                    [&](uint32_t e) -> C2& { return line[e]; }, gbar, scratch);
          }
        } else if (P.type == PASS_COL) {
          const uint32_t nrep = nrep_f();
          for (uint32_t b = rep_f() + nrep * (grp * K + rank); b < Cb; b += nrep * K * ngrp) {
            const uint32_t lstr = ldm<G>(strB + b);
            if (K == 1) {
              group_line_ops<R, A, G>(ops, I.coef, pool, P.op0, P.op1, rev, Ca, lstr, gt, gthreads,
                                      [&](uint32_t e) -> C2& { return blk[(size_t)e * Cb + b]; }, gbar, scratch);
            } else {
              auto ok = [](uint32_t) { return true; };
              auto remote = [&](uint32_t i) { return at(i, b); };
              auto local = [&](uint32_t i) { return stage + i; };
              group_copy<C2, kDepth>(Ca, gt, gthreads, ok, remote, local);
              gbar();
              group_line_ops<R, A, G>(ops, I.coef, pool, P.op0, P.op1, rev, Ca, lstr, gt, gthreads,
                                      [&](uint32_t e) -> C2& { return stage[e]; }, gbar, scratch);
              group_copy<C2, kDepth>(Ca, gt, gthreads, ok, local, remote);
              gbar();
            }
          }
        } else {  // PASS_MIX: one column pair per group tile
          const uint2* __restrict__ mt = reinterpret_cast<const uint2*>(pool + P.mixtab);
          for (uint32_t tile = grp * K + rank; tile < P.mixcount; tile += K * ngrp) {
            const uint2 pr = ldm<G>(mt + tile);
            const uint32_t b01 = pr.x & 0x7fffffffu, b10 = pr.y, pb = pr.x >> 31;
            auto parb = [&](uint32_t) { return pb; };
            if (K == 1) {
              auto left = [&](uint32_t, uint32_t a) -> C2& { return blk[(size_t)a * Cb + b01]; };
              auto right = [&](uint32_t, uint32_t a) -> C2& { return blk[(size_t)a * Cb + b10]; };
              group_mix_ops<R, A, G>(ops, I.coef, pool, P.op0, P.op1, rev, 0, 1, gt, gthreads, left, right, parb,
                                     gbar, scratch);
            } else {
              // element i: row i >> 1, side i & 1 (gthreads is even: a thread's side is fixed)
              const uint32_t mycol = (gt & 1) ? b10 : b01;
              auto ok = [](uint32_t) { return true; };
              auto remote = [&](uint32_t i) { return at(i >> 1, mycol); };
              auto local = [&](uint32_t i) { return stage + i; };
              group_copy<C2, kDepth>(Ca << 1, gt, gthreads, ok, remote, local);
              gbar();
              auto left = [&](uint32_t, uint32_t a) -> C2& { return stage[2 * a]; };
              auto right = [&](uint32_t, uint32_t a) -> C2& { return stage[2 * a + 1]; };
              group_mix_ops<R, A, G>(ops, I.coef, pool, P.op0, P.op1, rev, 0, 1, gt, gthreads, left, right, parb,
                                     gbar, scratch);
              group_copy<C2, kDepth>(Ca << 1, gt, gthreads, ok, local, remote);
              gbar();
            }
          }
        }
        if (in_group) wp_fetch(next_pi);
        barrier();
        if (P.type != PASS_MIX && nrep_f() > 1) {
          exchange(P.type == PASS_COL);
          barrier();
        }
        pj += span - 1;
      }
    }
    if (rep_f() == 0) {
      C2* dst = gstate + (uint64_t)(I.in_place ? I.first : k) * ld + (uint64_t)row0 * Cb;
      for (uint32_t i = threadIdx.x; i < nown; i += blockDim.x) dst[i] = blk[i];
    }
    barrier();
  }
  asm volatile("cp.async.wait_all;" ::: "memory");
}

template <typename R, class A, bool MS>
static cudaError_t launch_res(const ResidentLaunch& rl, cudaStream_t s) {
  const uint32_t nrep = rl.group == 3 && rl.cluster > 1 && rl.replicas > 1 ? rl.replicas : 1u;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(rl.ninst * nrep * rl.cluster);
  cfg.blockDim = dim3(32 * rl.warps_per_cta);
  cfg.dynamicSmemBytes = rl.smem_bytes;
  cfg.stream = s;
  cudaLaunchAttribute at[2];
  at[0].id = cudaLaunchAttributeClusterDimension;
  at[0].val.clusterDim.x = rl.cluster;
  at[0].val.clusterDim.y = 1;
  at[0].val.clusterDim.z = 1;
  // replicas wait on one another: they must all be resident at once
  at[1].id = cudaLaunchAttributeCooperative;
  at[1].val.cooperative = 1;
  cfg.attrs = at;
  cfg.numAttrs = nrep > 1 ? 2 : 1;
  auto kern = rl.group == 1 ? k_resident_group<R, A, MS>
                            : (rl.group == 2 ? k_resident<R, A, MS, true>
                                             : (rl.group == 3 ? (nrep > 1 ? k_resident_lean<R, A, MS, true>
                                                                          : k_resident_lean<R, A, MS, false>)
                                                              : k_resident<R, A, MS, false>));
  cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)rl.smem_bytes);
  if (e) return e;
  if (rl.cluster > 8) {
    e = cudaFuncSetAttribute(kern, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
    if (e) return e;
  }
  e = cudaLaunchKernelEx(&cfg, kern, rl.insts, rl.stage_elems);
  return e;
}

template <bool MS>
static cudaError_t launch_resident_ms(const ResidentLaunch& rl, int dtype, int exact, cudaStream_t s) {
  if (dtype == QPE_C128) {
    if (exact) return launch_res<double, ExactD, MS>(rl, s);
    return launch_res<double, Fast<double>, MS>(rl, s);
  }
  return launch_res<float, Fast<float>, MS>(rl, s);
}

cudaError_t launch_resident(const ResidentLaunch& rl, int dtype, int exact, cudaStream_t s) {
  return rl.meta_smem ? launch_resident_ms<true>(rl, dtype, exact, s) : launch_resident_ms<false>(rl, dtype, exact, s);
}

template <typename R, class A, bool MS>
static cudaError_t carveout_t(int percent) {
  cudaError_t e = cudaFuncSetAttribute(k_resident<R, A, MS, false>, cudaFuncAttributePreferredSharedMemoryCarveout, percent);
  if (e) return e;
  e = cudaFuncSetAttribute(k_resident<R, A, MS, true>, cudaFuncAttributePreferredSharedMemoryCarveout, percent);
  if (e) return e;
  e = cudaFuncSetAttribute(k_resident_lean<R, A, MS, false>, cudaFuncAttributePreferredSharedMemoryCarveout, percent);
  if (e) return e;
  e = cudaFuncSetAttribute(k_resident_lean<R, A, MS, true>, cudaFuncAttributePreferredSharedMemoryCarveout, percent);
  if (e) return e;
  return cudaFuncSetAttribute(k_resident_group<R, A, MS>, cudaFuncAttributePreferredSharedMemoryCarveout, percent);
}

template <bool MS>
static cudaError_t carveout_ms(int dtype, int exact, int percent) {
  if (dtype == QPE_C128) {
    if (exact) return carveout_t<double, ExactD, MS>(percent);
    return carveout_t<double, Fast<double>, MS>(percent);
  }
  return carveout_t<float, Fast<float>, MS>(percent);
}

cudaError_t set_resident_carveout(int dtype, int exact, int percent) {
  cudaError_t e = carveout_ms<false>(dtype, exact, percent);
  if (e) return e;
  return carveout_ms<true>(dtype, exact, percent);
}


}  // namespace qpe
