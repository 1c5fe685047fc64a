// mlp.cu - the learned initial-state model on Blackwell tensor cores.
//
// An MLP over occupation bit strings proposes the amplitudes of the QPE initial
// state: input the n_bits occupations (0 / 1, zero-padded to 64 features), three
// hidden layers of 256 with GELU, output (log|a|, phase). Weights and
// activations are BF16, every product is accumulated in FP32 in tensor memory;
// master weights, Adam moments, biases and the loss are FP32.
//
// Every matrix product is one tcgen05 GEMM kernel (k_gemm): D[M, N] = A[M, K] .
// B[N, K]^T with A and B K-major BF16 in global memory, tiles of 128 x BN
// (BN = 16, 64 or 256) per CTA. One thread issues the TMA loads of a 4-stage
// ring and the MMAs (M = 128, N = BN, K = 16 each) into a TMEM accumulator; the
// four warps then read the accumulator with tcgen05.ld and apply the fused
// epilogue (bias + GELU with the pre-activation kept for the backward pass, the
// GELU derivative for the backward pass, or a plain FP32 store).
//
// A training step is forward (4 GEMMs), loss, backward through the activations
// (3 GEMMs with the GELU derivative fused), weight gradients (4 GEMMs over the
// batch, operands transposed by k_transpose), bias gradients and Adam.
#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <cudaTypedefs.h>
#include <stdint.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <mutex>
#include <vector>

#include "../../include/qpe_gb300_mlp.h"
#include "abi_internal.h"
#include "umma.cuh"

namespace qpe {

using bf16 = __nv_bfloat16;

enum GemmEpi : int { EPI_F32 = 0, EPI_BIAS_GELU = 1, EPI_DGELU = 2, EPI_BIAS_F32 = 3 };

struct GemmArgs {
  uint32_t M, N, K;
  const float* bias;     // EPI_BIAS_*: [N]
  void* out;             // FP32 (EPI_F32, EPI_BIAS_F32) or BF16 (EPI_BIAS_GELU, EPI_DGELU), row stride ldo
  uint32_t ldo;
  float* pre_out;        // EPI_BIAS_GELU: pre-activation, FP32, stride ldo
  const float* pre_in;   // EPI_DGELU: the forward pre-activation, FP32, stride ldo
  int* err;              // set when a wait runs out
  uint32_t ksplit;       // EPI_F32: CTAs along K (grid z); slice z writes out + z * split_stride
  size_t split_stride;
  bf16* out_t;           // BF16 epilogues: if set, the output transposed as well ([N, M], row stride ldt),
  uint32_t ldt;          //   the K-major operand of the weight-gradient product (no separate transpose)
};

constexpr uint32_t kStages = 4;
constexpr uint32_t kABytes = 128 * 128;  // 128 rows x 64 BF16

template <uint32_t BN>
constexpr size_t gemm_smem_bytes() {
  return 1024 + (size_t)kStages * (kABytes + BN * 128) + (2 * kStages + 1) * 8 + 16;
}

__device__ __forceinline__ float gelu(float x) { return 0.5f * x * (1.0f + erff(x * 0.70710678118654752f)); }
__device__ __forceinline__ float gelu_grad(float x) {
  return 0.5f * (1.0f + erff(x * 0.70710678118654752f)) + x * 0.39894228040143268f * expf(-0.5f * x * x);
}

template <int EPI, uint32_t BN>
__global__ void __launch_bounds__(128, 1)
    k_gemm(const __grid_constant__ CUtensorMap ta, const __grid_constant__ CUtensorMap tb, GemmArgs g) {
  constexpr uint32_t kBBytes = BN * 128;
  constexpr uint32_t kStage = kABytes + kBBytes;
  constexpr uint32_t kCols = BN < 32 ? 32 : BN;
  extern __shared__ uint8_t smem_raw[];
  const uint32_t raw = umma::smem_u32(smem_raw);
  const uint32_t base = (raw + 1023u) & ~1023u;  // 128-byte swizzle atoms want 1024-byte alignment
  uint8_t* basep = smem_raw + (base - raw);
  const uint32_t bars = base + kStages * kStage;
  auto full = [&](uint32_t s) { return bars + 8 * s; };
  auto empty = [&](uint32_t s) { return bars + 8 * (kStages + s); };
  const uint32_t done = bars + 8 * (2 * kStages);
  uint32_t* slot = reinterpret_cast<uint32_t*>(basep + kStages * kStage + (2 * kStages + 1) * 8);
  const uint32_t warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const uint32_t m0 = blockIdx.y * 128, n0 = blockIdx.x * BN;
  // k-blocks of this CTA's K slice (all of K unless split)
  const uint32_t nk_all = g.K / 64, ks = g.ksplit ? g.ksplit : 1u;
  const uint32_t kb0 = (uint32_t)((uint64_t)nk_all * blockIdx.z / ks);
  const uint32_t nk = (uint32_t)((uint64_t)nk_all * (blockIdx.z + 1) / ks) - kb0;

  if (threadIdx.x == 0) {
    for (uint32_t s = 0; s < kStages; ++s) {
      umma::mbar_init(full(s), 1);
      umma::mbar_init(empty(s), 1);
    }
    umma::mbar_init(done, 1);
    umma::fence_barrier_init();
  }
  __syncwarp();
  if (warp == 0) umma::tmem_alloc(umma::smem_u32(slot), kCols);
  umma::fence_before_sync();
  __syncthreads();
  umma::fence_after_sync();
  const uint32_t tmem = *slot;

  if (threadIdx.x == 0) {
    auto issue = [&](uint32_t kb, uint32_t s) {
      const uint32_t a = base + s * kStage;
      umma::mbar_expect_tx(full(s), kStage);
      umma::tma_load_2d(a, &ta, (int32_t)((kb0 + kb) * 64), (int32_t)m0, full(s));
      umma::tma_load_2d(a + kABytes, &tb, (int32_t)((kb0 + kb) * 64), (int32_t)n0, full(s));
    };
    const uint32_t idesc = umma::idesc_bf16(128, BN);
    uint32_t issued = 0, kb = 0;
    bool ok = true;
    for (; issued < nk && issued < kStages; ++issued) issue(issued, issued);
    for (; kb < nk; ++kb) {
      const uint32_t s = kb % kStages, ph = (kb / kStages) & 1;
      if (!umma::mbar_wait(full(s), ph)) {
        ok = false;
        break;
      }
      umma::fence_after_sync();
      const uint32_t a = base + s * kStage, b = a + kABytes;
#pragma unroll
      for (uint32_t k = 0; k < 4; ++k)
        umma::mma_bf16(tmem, umma::sdesc_k128(a + 32 * k), umma::sdesc_k128(b + 32 * k), idesc, (kb | k) != 0);
      umma::mma_commit(empty(s));
      if (kb + kStages < nk) {
        if (!umma::mbar_wait(empty(s), ph)) {
          ok = false;
          break;
        }
        issue(kb + kStages, s);
        ++issued;
      }
    }
    umma::mma_commit(done);
    if (!ok) {
      atomicExch(g.err, 1);
      // Let the loads still in flight land before the CTA leaves.
      for (uint32_t j = kb; j < issued; ++j) umma::mbar_wait(full(j % kStages), (j / kStages) & 1, 1u << 16);
    }
  }
  __syncwarp();

  // Epilogue: warp w owns accumulator lanes (rows) 32 w .. 32 w + 31.
  const bool ready = umma::mbar_wait(done, 0);
  umma::fence_after_sync();
  if (!ready && lane == 0) atomicExch(g.err, 2);
  const uint32_t row = m0 + warp * 32 + lane;
  for (uint32_t c = 0; c < BN; c += 16) {
    float v[16];
    umma::tmem_ld16(tmem + ((warp * 32u) << 16) + c, v);
    if (!ready || row >= g.M) continue;
    const uint32_t col = n0 + c;
    const size_t off = (size_t)row * g.ldo + col;
    if (EPI == EPI_F32 || EPI == EPI_BIAS_F32) {
      float4* o = reinterpret_cast<float4*>(reinterpret_cast<float*>(g.out) + off + blockIdx.z * g.split_stride);
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        float4 x = make_float4(v[4 * q], v[4 * q + 1], v[4 * q + 2], v[4 * q + 3]);
        if (EPI == EPI_BIAS_F32) {
          x.x += g.bias[col + 4 * q];
          x.y += g.bias[col + 4 * q + 1];
          x.z += g.bias[col + 4 * q + 2];
          x.w += g.bias[col + 4 * q + 3];
        }
        o[q] = x;
      }
    } else {
      float x[16];
      if (EPI == EPI_BIAS_GELU) {
        float4* pre = reinterpret_cast<float4*>(g.pre_out + off);
#pragma unroll
        for (int i = 0; i < 16; ++i) x[i] = v[i] + g.bias[col + i];
#pragma unroll
        for (int q = 0; q < 4; ++q) pre[q] = make_float4(x[4 * q], x[4 * q + 1], x[4 * q + 2], x[4 * q + 3]);
#pragma unroll
        for (int i = 0; i < 16; ++i) x[i] = gelu(x[i]);
      } else {
        const float4* pre = reinterpret_cast<const float4*>(g.pre_in + off);
#pragma unroll
        for (int q = 0; q < 4; ++q) {
          const float4 p = pre[q];
          x[4 * q] = v[4 * q] * gelu_grad(p.x);
          x[4 * q + 1] = v[4 * q + 1] * gelu_grad(p.y);
          x[4 * q + 2] = v[4 * q + 2] * gelu_grad(p.z);
          x[4 * q + 3] = v[4 * q + 3] * gelu_grad(p.w);
        }
      }
      __align__(16) bf16 h[16];
#pragma unroll
      for (int i = 0; i < 16; ++i) h[i] = __float2bfloat16_rn(x[i]);
      uint4* o = reinterpret_cast<uint4*>(reinterpret_cast<bf16*>(g.out) + off);
      o[0] = reinterpret_cast<const uint4*>(h)[0];
      o[1] = reinterpret_cast<const uint4*>(h)[1];
      if (g.out_t) {
        // a warp's 32 lanes hold 32 consecutive rows: each transposed column is
        // one 64-byte run
#pragma unroll
        for (int i = 0; i < 16; ++i) g.out_t[(size_t)(col + i) * g.ldt + row] = h[i];
      }
    }
  }
  umma::fence_before_sync();
  __syncthreads();
  if (warp == 0) umma::tmem_dealloc(tmem, kCols);
}

// ---- small kernels of the training step ---------------------------------------

// out[r, c] = sum over slices z (in order) of part[z][r, c]: the fixed-order
// reduction of a split-K product (rows x cols, row stride ld in both).
__global__ void k_reduce_split(const float* __restrict__ part, uint32_t ks, size_t stride, uint32_t rows,
                               uint32_t cols, uint32_t ld, float* __restrict__ out, uint32_t ldo) {
  const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (size_t)rows * cols) return;
  const size_t r = i / cols, c = i - r * cols;
  float s = 0.f;
  for (uint32_t z = 0; z < ks; ++z) s += part[z * stride + r * ld + c];
  out[r * ldo + c] = s;
}


// dst[C, R] = src[R, C]^T (BF16), 32 x 32 tiles through shared memory.
__global__ void k_transpose(const bf16* __restrict__ src, bf16* __restrict__ dst, uint32_t R, uint32_t C,
                            uint32_t lds, uint32_t ldd) {
  __shared__ bf16 t[32][33];
  const uint32_t r0 = blockIdx.y * 32, c0 = blockIdx.x * 32;
  for (uint32_t i = threadIdx.y; i < 32; i += blockDim.y) {
    const uint32_t r = r0 + i, c = c0 + threadIdx.x;
    t[i][threadIdx.x] = (r < R && c < C) ? src[(size_t)r * lds + c] : __float2bfloat16_rn(0.f);
  }
  __syncthreads();
  for (uint32_t i = threadIdx.y; i < 32; i += blockDim.y) {
    const uint32_t c = c0 + i, r = r0 + threadIdx.x;
    if (c < C && r < R) dst[(size_t)c * ldd + r] = t[threadIdx.x][i];
  }
}

__device__ __forceinline__ uint64_t mix64(uint64_t x) {
  x ^= x >> 30;
  x *= 0xbf58476d1ce4e5b9ull;
  x ^= x >> 27;
  x *= 0x94d049bb133111ebull;
  x ^= x >> 31;
  return x;
}

// Row b of the batch: sample idx (random when `sample`, else b) -> input
// features (bit j of the occupation string as 0 / 1 for j < n_bits, then the
// sample's n_feat extra features, zero past them) and the sample's targets. Rows
// past `count` are zero with weight 0.
__global__ void k_gather_batch(const uint64_t* __restrict__ bits, const float* __restrict__ feats, uint32_t n_feat,
                               const float* __restrict__ tla, const float* __restrict__ tph,
                               const float* __restrict__ tw, uint64_t nsamples, uint32_t count, uint32_t Bp,
                               uint32_t n_bits, int sample, uint64_t seed, const uint64_t* __restrict__ step,
                               bf16* __restrict__ X0, float* __restrict__ bla, float* __restrict__ bph,
                               float* __restrict__ bw) {
  const uint32_t b = blockIdx.x;
  if (b >= Bp) return;
  uint64_t idx = b;
  const bool live = b < count;
  if (live && sample) idx = mix64(seed ^ mix64(*step * 0x9e3779b97f4a7c15ull + b)) % nsamples;
  const uint64_t x = live ? bits[idx] : 0ull;
  for (uint32_t j = threadIdx.x; j < 64; j += blockDim.x) {
    float v = 0.f;
    if (live && j < n_bits) v = ((x >> j) & 1ull) ? 1.f : 0.f;
    else if (live && j < n_bits + n_feat) v = feats[idx * n_feat + (j - n_bits)];
    X0[(size_t)b * 64 + j] = __float2bfloat16_rn(v);
  }
  if (threadIdx.x == 0) {
    bla[b] = live && tla ? tla[idx] : 0.f;
    bph[b] = live && tph ? tph[idx] : 0.f;
    bw[b] = live && tw ? tw[idx] : 0.f;
  }
}

// Loss (1 / count) sum_b w_b [(la_b - t_b)^2 + (1 - cos(ph_b - p_b))] and its
// gradient into columns 0, 1 of dY (BF16, stride 64; the other columns stay 0).
__global__ void k_loss(const float* __restrict__ Y, const float* __restrict__ bla, const float* __restrict__ bph,
                       const float* __restrict__ bw, uint32_t count, uint32_t Bp, bf16* __restrict__ dY,
                       float* __restrict__ loss) {
  __shared__ float red[256];
  const uint32_t b = blockIdx.x * blockDim.x + threadIdx.x;
  float l = 0.f;
  if (b < Bp) {
    float g0 = 0.f, g1 = 0.f;
    if (b < count) {
      const float inv = 1.0f / (float)count;
      const float w = bw[b], dl = Y[(size_t)b * 16] - bla[b], dp = Y[(size_t)b * 16 + 1] - bph[b];
      l = w * (dl * dl + (1.0f - cosf(dp))) * inv;
      g0 = 2.0f * w * dl * inv;
      g1 = w * sinf(dp) * inv;
    }
    dY[(size_t)b * 64] = __float2bfloat16_rn(g0);
    dY[(size_t)b * 64 + 1] = __float2bfloat16_rn(g1);
  }
  red[threadIdx.x] = l;
  __syncthreads();
  for (uint32_t s = blockDim.x / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) red[threadIdx.x] += red[threadIdx.x + s];
    __syncthreads();
  }
  if (threadIdx.x == 0) atomicAdd(loss, red[0]);
}

constexpr uint32_t kColsumRows = 64;

// Column sums of a [R x C] BF16 matrix (row stride lds, C and lds even) in two
// fixed-order phases: k_colsum_part writes one partial row per kColsumRows rows
// (each thread two columns, four independent accumulators over rows r = j mod 4),
// k_colsum_final adds the partial rows of a column in a fixed tree.
__global__ void k_colsum_part(const bf16* __restrict__ src, uint32_t R, uint32_t C, uint32_t lds,
                              float* __restrict__ part) {
  const uint32_t c = 2 * threadIdx.x, r0 = blockIdx.x * kColsumRows;
  if (c >= C) return;
  const uint32_t r1 = min(R, r0 + kColsumRows);
  float2 a[4] = {};
  for (uint32_t r = r0; r < r1; r += 4) {
#pragma unroll
    for (uint32_t j = 0; j < 4; ++j) {
      if (r + j < r1) {
        const float2 v = __bfloat1622float2(*reinterpret_cast<const __nv_bfloat162*>(src + (size_t)(r + j) * lds + c));
        a[j].x += v.x;
        a[j].y += v.y;
      }
    }
  }
  part[(size_t)blockIdx.x * C + c] = (a[0].x + a[1].x) + (a[2].x + a[3].x);
  part[(size_t)blockIdx.x * C + c + 1] = (a[0].y + a[1].y) + (a[2].y + a[3].y);
}
__global__ void k_colsum_final(const float* __restrict__ part, uint32_t nparts, uint32_t C, float* __restrict__ out) {
  __shared__ float red[4];
  const uint32_t c = blockIdx.x;  // one CTA of 128 threads per column
  float s = 0.f;
  for (uint32_t p = threadIdx.x; p < nparts; p += blockDim.x) s += part[(size_t)p * C + c];
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x == 0) out[c] = (red[0] + red[1]) + (red[2] + red[3]);
}

// One parameter block of the Adam step: its offset in the parameter, moment and
// gradient arrays (the gradient block has the same layout), its shape, and the
// BF16 copy (rows x cols, stride ldb) and transpose (cols x rows, stride ldt)
// it refreshes (null: none).
struct AdamBlock {
  uint32_t off, rows, cols, ldb, ldt;
  bf16* wb;
  bf16* wt;
};
constexpr int kAdamBlocks = 8;
struct AdamBlocks {
  AdamBlock b[kAdamBlocks];
  uint32_t start[kAdamBlocks + 1];  // flattened element index of each block's first element
};

// Adam over every parameter block in one launch: thread i updates flattened
// element i, finds its block from `start`, and writes the block's BF16 copy and
// transpose.
__global__ void k_adam(float* __restrict__ w, float* __restrict__ m, float* __restrict__ v,
                       const float* __restrict__ grad, const __grid_constant__ AdamBlocks blocks, float lr, float b1,
                       float b2, float eps, float c1, float c2) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= blocks.start[kAdamBlocks]) return;
  int k = 0;
#pragma unroll
  for (int q = 1; q < kAdamBlocks; ++q) k += i >= blocks.start[q] ? 1 : 0;
  const AdamBlock& B = blocks.b[k];
  const uint32_t e = i - blocks.start[k], r = e / B.cols, c = e - r * B.cols;
  const size_t o = (size_t)B.off + e;
  const float gr = grad[o];
  const float mi = b1 * m[o] + (1.f - b1) * gr;
  const float vi = b2 * v[o] + (1.f - b2) * gr * gr;
  m[o] = mi;
  v[o] = vi;
  const float wi = w[o] - lr * (mi * c1) / (sqrtf(vi * c2) + eps);
  w[o] = wi;
  if (B.wb) B.wb[(size_t)r * B.ldb + c] = __float2bfloat16_rn(wi);
  if (B.wt) B.wt[(size_t)c * B.ldt + r] = __float2bfloat16_rn(wi);
}

__global__ void k_cast_bf16(const float* __restrict__ w, uint32_t rows, uint32_t cols, bf16* __restrict__ wb,
                            uint32_t ldb, bf16* __restrict__ wt, uint32_t ldt) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= rows * cols) return;
  const uint32_t r = i / cols, c = i - r * cols;
  if (wb) wb[(size_t)r * ldb + c] = __float2bfloat16_rn(w[i]);
  if (wt) wt[(size_t)c * ldt + r] = __float2bfloat16_rn(w[i]);
}

__global__ void k_add_u64(uint64_t* p, uint64_t v) { *p += v; }

// ---- host side -----------------------------------------------------------------

static PFN_cuTensorMapEncodeTiled_v12000 encode_fn() {
  static std::once_flag once;
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  std::call_once(once, [] {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
  });
  if (!fn) throw Error(QPE_ERR_CUDA, "cuTensorMapEncodeTiled is not available");
  return fn;
}

// Tensor map of a row-major BF16 matrix [rows, cols] (row stride ld elements),
// box 64 columns x box_rows rows, 128-byte swizzle.
static CUtensorMap make_map(const void* ptr, uint64_t rows, uint64_t cols, uint64_t ld, uint32_t box_rows) {
  if ((reinterpret_cast<uintptr_t>(ptr) & 15) || (ld * 2) % 16 || cols % 64 || box_rows > 256 || rows < box_rows)
    throw Error(QPE_ERR_INVALID, "tensor map: operand not aligned to the 64 x rows tile");
  CUtensorMap m;
  std::memset(&m, 0, sizeof(m));
  const cuuint64_t dims[2] = {cols, rows};
  const cuuint64_t strides[1] = {ld * 2};
  const cuuint32_t box[2] = {64, box_rows};
  const cuuint32_t es[2] = {1, 1};
  const CUresult r = encode_fn()(&m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<void*>(ptr), dims, strides, box,
                                 es, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                                 CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) throw Error(QPE_ERR_CUDA, "cuTensorMapEncodeTiled failed: " + std::to_string((int)r));
  return m;
}

// One GEMM: the operands' maps, the shape and the epilogue.
struct Gemm {
  CUtensorMap ta, tb;
  GemmArgs g;
  int epi;
  uint32_t bn;
  float* final_out = nullptr;  // split-K: the reduced product's destination
  uint32_t final_ldo = 0;
};

template <int EPI, uint32_t BN>
static cudaError_t launch_gemm_t(const Gemm& G, cudaStream_t s) {
  constexpr size_t smem = gemm_smem_bytes<BN>();
  cudaError_t e = cudaFuncSetAttribute(k_gemm<EPI, BN>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e) return e;
  const uint32_t ks = G.g.ksplit ? G.g.ksplit : 1u;
  k_gemm<EPI, BN><<<dim3(G.g.N / BN, G.g.M / 128, ks), 128, smem, s>>>(G.ta, G.tb, G.g);
  e = cudaGetLastError();
  if (e || ks == 1 || !G.final_out) return e;
  const size_t n = (size_t)G.g.M * G.g.N;
  k_reduce_split<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(reinterpret_cast<const float*>(G.g.out), ks,
                                                             G.g.split_stride, G.g.M, G.g.N, G.g.ldo, G.final_out,
                                                             G.final_ldo);
  return cudaGetLastError();
}

static cudaError_t launch_gemm(const Gemm& G, cudaStream_t s) {
#define QPE_GEMM_CASE(E, B) \
  if (G.epi == E && G.bn == B) return launch_gemm_t<E, B>(G, s);
  QPE_GEMM_CASE(EPI_F32, 16)
  QPE_GEMM_CASE(EPI_F32, 64)
  QPE_GEMM_CASE(EPI_F32, 256)
  QPE_GEMM_CASE(EPI_BIAS_F32, 16)
  QPE_GEMM_CASE(EPI_BIAS_GELU, 256)
  QPE_GEMM_CASE(EPI_DGELU, 256)
#undef QPE_GEMM_CASE
  return cudaErrorInvalidValue;
}

// Checks a GEMM's shape against its operands: A [M, K] with M % 128 == 0, B [N, K]
// with N % BN == 0, K % 64 == 0, output stride a multiple of 16 bytes.
static Gemm make_gemm(int epi, uint32_t bn, const void* A, uint32_t lda, const void* B, uint32_t ldb, uint32_t M,
                      uint32_t N, uint32_t K, void* out, uint32_t ldo, const float* bias, float* pre_out,
                      const float* pre_in, int* err) {
  if (M == 0 || M % 128 || N % bn || K == 0 || K % 64 || ldo % 8 || (N > ldo))
    throw Error(QPE_ERR_INVALID, "GEMM shape outside the tile grid");
  Gemm G;
  G.ta = make_map(A, M, K, lda, 128);
  G.tb = make_map(B, N, K, ldb, bn);
  G.g = GemmArgs{M, N, K, bias, out, ldo, pre_out, pre_in, err, 1u, 0, nullptr, 0};
  G.epi = epi;
  G.bn = bn;
  return G;
}

// A plain FP32 product split along K over enough CTAs to fill the GPU: the
// slices write partial tiles into `scratch` (ksplit x M x N) and a fixed-order
// reduction writes the result to out.
static Gemm make_gemm_splitk(uint32_t bn, const void* A, uint32_t lda, const void* B, uint32_t ldb, uint32_t M,
                             uint32_t N, uint32_t K, float* out, uint32_t ldo, float* scratch, size_t scratch_elems,
                             uint32_t num_sms, int* err) {
  const uint32_t tiles = (M / 128) * (N / bn), nk = K / 64;
  uint32_t ks = std::max(1u, std::min(nk, (num_sms + tiles - 1) / tiles));
  while (ks > 1 && (size_t)ks * M * N > scratch_elems) --ks;
  Gemm G = make_gemm(EPI_F32, bn, A, lda, B, ldb, M, N, K, ks > 1 ? scratch : out, ks > 1 ? N : ldo, nullptr,
                     nullptr, nullptr, err);
  G.g.ksplit = ks;
  G.g.split_stride = (size_t)M * N;
  if (ks > 1) {
    G.final_out = out;
    G.final_ldo = ldo;
  }
  return G;
}

}  // namespace qpe

using namespace qpe;

// ---- the model -----------------------------------------------------------------

struct qpe_mlp {
  qpe_context* ctx = nullptr;
  uint32_t n_bits = 0, n_feat = 0, Bp = 0;  // inputs: n_bits occupations, then n_feat features
  static constexpr uint32_t K0 = 64, H = 256, NO = 16;
  // FP32 master parameters, Adam moments and gradients, one flat array each.
  DevBuf params, mom1, mom2, grads;
  // BF16 weights (row-major [out, in]) and the transposes the backward pass reads.
  DevBuf W1b, W2b, W3b, W4b, W2t, W3t, W4t;
  // activations
  DevBuf X0, pre1, pre2, pre3, H1, H2, H3, Y, dY, dZ1, dZ2, dZ3;
  DevBuf X0T, H1T, H2T, H3T, dYT, dZ1T, dZ2T, dZ3T;
  DevBuf bla, bph, bw, loss, err, step, colpart, splitk;
  // training set
  DevBuf dbits, dfeat, dla, dph, dw;
  uint64_t nsamples = 0;
  std::vector<Gemm> fwd, bwd, wgrad;
  cudaGraphExec_t train_exec = nullptr;
  uint64_t train_seed = 0;
  float train_lr = 0.f;
  uint64_t adam_t = 0;
  double tensor_flops_per_step = 0;

  // Parameter block offsets in the flat arrays.
  static constexpr size_t oW1 = 0, ob1 = oW1 + (size_t)H * K0, oW2 = ob1 + H, ob2 = oW2 + (size_t)H * H,
                          oW3 = ob2 + H, ob3 = oW3 + (size_t)H * H, oW4 = ob3 + H, ob4 = oW4 + (size_t)NO * H,
                          nparams = ob4 + NO;
  ~qpe_mlp() {
    if (train_exec) cudaGraphExecDestroy(train_exec);
  }
};

namespace qpe {

static void mlp_alloc(qpe_mlp* m) {
  const size_t Bp = m->Bp, H = qpe_mlp::H, K0 = qpe_mlp::K0, NO = qpe_mlp::NO, b2 = sizeof(bf16);
  m->params.alloc(qpe_mlp::nparams * 4);
  m->mom1.alloc(qpe_mlp::nparams * 4);
  m->mom2.alloc(qpe_mlp::nparams * 4);
  m->grads.alloc((qpe_mlp::nparams + 128 * 256) * 4);
  m->W1b.alloc(H * K0 * b2);
  m->W2b.alloc(H * H * b2);
  m->W3b.alloc(H * H * b2);
  m->W4b.alloc(NO * H * b2);
  m->W2t.alloc(H * H * b2);
  m->W3t.alloc(H * H * b2);
  m->W4t.alloc(H * K0 * b2);  // [256, 64]: W4^T in columns 0..15, zero beyond
  m->X0.alloc(Bp * K0 * b2);
  for (DevBuf* p : {&m->pre1, &m->pre2, &m->pre3}) p->alloc(Bp * H * 4);
  for (DevBuf* p : {&m->H1, &m->H2, &m->H3, &m->dZ1, &m->dZ2, &m->dZ3}) p->alloc(Bp * H * b2);
  m->Y.alloc(Bp * NO * 4);
  m->dY.alloc(Bp * K0 * b2);
  m->X0T.alloc(K0 * Bp * b2);
  for (DevBuf* p : {&m->H1T, &m->H2T, &m->H3T, &m->dZ1T, &m->dZ2T, &m->dZ3T}) p->alloc(H * Bp * b2);
  m->dYT.alloc(128 * Bp * b2);  // 128 rows for the M = 128 tile; rows past 63 stay zero
  m->colpart.alloc(((Bp + kColsumRows - 1) / kColsumRows) * H * 4);
  const size_t splitk_elems = (size_t)64 * 256 * 256;  // up to 64 K slices of a 256 x 256 gradient
  m->splitk.alloc(splitk_elems * 4);
  m->bla.alloc(Bp * 4);
  m->bph.alloc(Bp * 4);
  m->bw.alloc(Bp * 4);
  m->loss.alloc(16);
  m->err.alloc(16);
  m->step.alloc(16);
  for (DevBuf* p : {&m->mom1, &m->mom2, &m->grads, &m->W4t, &m->dY, &m->dYT, &m->err, &m->step, &m->loss})
    QPE_CK(cudaMemset(p->p, 0, p->bytes));
  // GEMMs of one step.
  int* err = m->err.as<int>();
  float* P = m->params.as<float>();
  float* G = m->grads.as<float>();
  const uint32_t B = m->Bp;
  m->fwd = {
      make_gemm(EPI_BIAS_GELU, 256, m->X0.p, 64, m->W1b.p, 64, B, 256, 64, m->H1.p, 256, P + qpe_mlp::ob1,
                m->pre1.as<float>(), nullptr, err),
      make_gemm(EPI_BIAS_GELU, 256, m->H1.p, 256, m->W2b.p, 256, B, 256, 256, m->H2.p, 256, P + qpe_mlp::ob2,
                m->pre2.as<float>(), nullptr, err),
      make_gemm(EPI_BIAS_GELU, 256, m->H2.p, 256, m->W3b.p, 256, B, 256, 256, m->H3.p, 256, P + qpe_mlp::ob3,
                m->pre3.as<float>(), nullptr, err),
      make_gemm(EPI_BIAS_F32, 16, m->H3.p, 256, m->W4b.p, 256, B, 16, 256, m->Y.p, 16, P + qpe_mlp::ob4, nullptr,
                nullptr, err)};
  m->bwd = {
      make_gemm(EPI_DGELU, 256, m->dY.p, 64, m->W4t.p, 64, B, 256, 64, m->dZ3.p, 256, nullptr, nullptr,
                m->pre3.as<float>(), err),
      make_gemm(EPI_DGELU, 256, m->dZ3.p, 256, m->W3t.p, 256, B, 256, 256, m->dZ2.p, 256, nullptr, nullptr,
                m->pre2.as<float>(), err),
      make_gemm(EPI_DGELU, 256, m->dZ2.p, 256, m->W2t.p, 256, B, 256, 256, m->dZ1.p, 256, nullptr, nullptr,
                m->pre1.as<float>(), err)};
  // the BF16 epilogues also write the transposed activations the weight-gradient
  // products read (H1..H3 and dZ1..dZ3, [256, B])
  m->fwd[0].g.out_t = m->H1T.as<bf16>();
  m->fwd[1].g.out_t = m->H2T.as<bf16>();
  m->fwd[2].g.out_t = m->H3T.as<bf16>();
  m->bwd[0].g.out_t = m->dZ3T.as<bf16>();
  m->bwd[1].g.out_t = m->dZ2T.as<bf16>();
  m->bwd[2].g.out_t = m->dZ1T.as<bf16>();
  for (Gemm* g : {&m->fwd[0], &m->fwd[1], &m->fwd[2], &m->bwd[0], &m->bwd[1], &m->bwd[2]}) g->g.ldt = B;
  // dW4 is [128, 256] over the padded dY^T, stored past the parameter blocks;
  // its rows 0..15 are copied into the W4 block.
  const uint32_t sms = (uint32_t)m->ctx->num_sms;
  float* sk = m->splitk.as<float>();
  m->wgrad = {make_gemm_splitk(64, m->dZ1T.p, B, m->X0T.p, B, 256, 64, B, G + qpe_mlp::oW1, 64, sk, splitk_elems,
                               sms, err),
              make_gemm_splitk(256, m->dZ2T.p, B, m->H1T.p, B, 256, 256, B, G + qpe_mlp::oW2, 256, sk, splitk_elems,
                               sms, err),
              make_gemm_splitk(256, m->dZ3T.p, B, m->H2T.p, B, 256, 256, B, G + qpe_mlp::oW3, 256, sk, splitk_elems,
                               sms, err),
              make_gemm_splitk(256, m->dYT.p, B, m->H3T.p, B, 128, 256, B, G + qpe_mlp::nparams, 256, sk,
                               splitk_elems, sms, err)};
  const double Bd = (double)B;
  m->tensor_flops_per_step = 2.0 * Bd * (256.0 * 64 + 2 * 256.0 * 256 + 16.0 * 256)      // forward
                             + 2.0 * Bd * (256.0 * 64 + 2 * 256.0 * 256)                  // backward data
                             + 2.0 * Bd * (256.0 * 64 + 2 * 256.0 * 256 + 128.0 * 256);  // weight gradients
}

static void cast_all(qpe_mlp* m, cudaStream_t s) {
  const float* P = m->params.as<float>();
  auto cast = [&](size_t off, uint32_t rows, uint32_t cols, void* wb, uint32_t ldb, void* wt, uint32_t ldt) {
    k_cast_bf16<<<(rows * cols + 255) / 256, 256, 0, s>>>(P + off, rows, cols, (bf16*)wb, ldb, (bf16*)wt, ldt);
  };
  cast(qpe_mlp::oW1, 256, 64, m->W1b.p, 64, nullptr, 0);
  cast(qpe_mlp::oW2, 256, 256, m->W2b.p, 256, m->W2t.p, 256);
  cast(qpe_mlp::oW3, 256, 256, m->W3b.p, 256, m->W3t.p, 256);
  cast(qpe_mlp::oW4, 16, 256, m->W4b.p, 256, m->W4t.p, 64);
  QPE_CK(cudaGetLastError());
}

// Forward pass of rows [0, count) of X0 (already built).
static void forward(qpe_mlp* m, cudaStream_t s) {
  for (const Gemm& g : m->fwd) QPE_CK(launch_gemm(g, s));
}

// Loss, backward and the gradients of every parameter into m->grads (W4 rows
// 0..15 and the bias sums copied into their blocks).
static void backward(qpe_mlp* m, uint32_t count, cudaStream_t s, float* loss) {
  const uint32_t B = m->Bp;
  k_loss<<<(B + 255) / 256, 256, 0, s>>>(m->Y.as<float>(), m->bla.as<float>(), m->bph.as<float>(),
                                         m->bw.as<float>(), count, B, m->dY.as<bf16>(), loss);
  QPE_CK(cudaGetLastError());
  for (const Gemm& g : m->bwd) QPE_CK(launch_gemm(g, s));
  const dim3 tb(32, 8);
  auto tr = [&](const DevBuf& src, uint32_t R, uint32_t C, uint32_t lds, DevBuf& dst, uint32_t ldd) {
    k_transpose<<<dim3((C + 31) / 32, (R + 31) / 32), tb, 0, s>>>(src.as<bf16>(), dst.as<bf16>(), R, C, lds, ldd);
  };
  // H1..H3 and dZ1..dZ3 were written transposed by their GEMMs' epilogues
  tr(m->X0, B, 64, 64, m->X0T, B);
  tr(m->dY, B, 64, 64, m->dYT, B);
  QPE_CK(cudaGetLastError());
  for (const Gemm& g : m->wgrad) QPE_CK(launch_gemm(g, s));
  float* G = m->grads.as<float>();
  QPE_CK(cudaMemcpyAsync(G + qpe_mlp::oW4, G + qpe_mlp::nparams, 16 * 256 * 4, cudaMemcpyDeviceToDevice, s));
  const uint32_t nparts = (B + kColsumRows - 1) / kColsumRows;
  auto colsum = [&](const DevBuf& src, uint32_t C, uint32_t lds, float* out) {
    k_colsum_part<<<nparts, 128, 0, s>>>(src.as<bf16>(), B, C, lds, m->colpart.as<float>());
    k_colsum_final<<<C, 128, 0, s>>>(m->colpart.as<float>(), nparts, C, out);
  };
  colsum(m->dZ1, 256, 256, G + qpe_mlp::ob1);
  colsum(m->dZ2, 256, 256, G + qpe_mlp::ob2);
  colsum(m->dZ3, 256, 256, G + qpe_mlp::ob3);
  colsum(m->dY, 16, 64, G + qpe_mlp::ob4);
  QPE_CK(cudaGetLastError());
}

static void adam(qpe_mlp* m, float lr, cudaStream_t s, float c1, float c2) {
  float* P = m->params.as<float>();
  float* M1 = m->mom1.as<float>();
  float* M2 = m->mom2.as<float>();
  float* G = m->grads.as<float>();
  // only the two live outputs of the last layer train; the padding stays zero
  const AdamBlock list[kAdamBlocks] = {
      {qpe_mlp::oW1, 256, 64, 64, 0, (bf16*)m->W1b.p, nullptr},
      {qpe_mlp::ob1, 1, 256, 0, 0, nullptr, nullptr},
      {qpe_mlp::oW2, 256, 256, 256, 256, (bf16*)m->W2b.p, (bf16*)m->W2t.p},
      {qpe_mlp::ob2, 1, 256, 0, 0, nullptr, nullptr},
      {qpe_mlp::oW3, 256, 256, 256, 256, (bf16*)m->W3b.p, (bf16*)m->W3t.p},
      {qpe_mlp::ob3, 1, 256, 0, 0, nullptr, nullptr},
      {qpe_mlp::oW4, 2, 256, 256, 64, (bf16*)m->W4b.p, (bf16*)m->W4t.p},
      {qpe_mlp::ob4, 1, 2, 0, 0, nullptr, nullptr}};
  AdamBlocks ab{};
  uint32_t total = 0;
  for (int k = 0; k < kAdamBlocks; ++k) {
    ab.b[k] = list[k];
    ab.start[k] = total;
    total += list[k].rows * list[k].cols;
  }
  ab.start[kAdamBlocks] = total;
  k_adam<<<(total + 255) / 256, 256, 0, s>>>(P, M1, M2, G, ab, lr, 0.9f, 0.999f, 1e-8f, c1, c2);
  QPE_CK(cudaGetLastError());
}

static void check_err(qpe_mlp* m) {
  int e = 0;
  QPE_CK(cudaMemcpy(&e, m->err.p, sizeof(int), cudaMemcpyDeviceToHost));
  if (e) throw Error(QPE_ERR_TIMEOUT, "tensor-core GEMM: a pipeline wait ran out (code " + std::to_string(e) + ")");
}

// The bounded wait every tcgen05 / TMA pipeline wait of this file uses
// (umma::mbar_wait), run alone on one mbarrier with nothing in flight: thread 0
// initialises it for one arrival and, if `arrive`, arrives; then every thread
// waits for phase 0 with `max_tries` polls. A wait that runs out sets *err and
// the kernel returns, as the GEMM kernels do.
__global__ void k_wait_probe(uint32_t max_tries, int arrive, int* err) {
  __shared__ __align__(8) uint64_t bar;
  const uint32_t b = umma::smem_u32(&bar);
  if (threadIdx.x == 0) {
    umma::mbar_init(b, 1);
    umma::fence_barrier_init();
  }
  __syncthreads();
  if (arrive && threadIdx.x == 0) asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(b) : "memory");
  if (!umma::mbar_wait(b, 0, max_tries)) atomicOr(err, 1);
}

static void use_ctx(qpe_context* ctx) {
  if (!ctx) throw Error(QPE_ERR_INVALID, "null context");
  QPE_CK(cudaSetDevice(ctx->device));
}

}  // namespace qpe

extern "C" {

int qpe_mlp_create(qpe_context* ctx, uint32_t n_bits, uint32_t batch, uint64_t seed, qpe_mlp** out) {
  return qpe_mlp_create2(ctx, n_bits, 0, batch, seed, out);
}

int qpe_mlp_create2(qpe_context* ctx, uint32_t n_bits, uint32_t n_feat, uint32_t batch, uint64_t seed,
                    qpe_mlp** out) {
  return guard([&] {
    use_ctx(ctx);
    if (!out) throw Error(QPE_ERR_INVALID, "null output");
    if (n_bits == 0 || n_bits > 64) throw Error(QPE_ERR_INVALID, "n_bits must be in 1..64");
    if (n_feat > 64 - n_bits) throw Error(QPE_ERR_INVALID, "n_bits + n_feat must be at most 64");
    if (batch == 0 || batch % 128 || batch > (1u << 20)) throw Error(QPE_ERR_INVALID, "batch must be a multiple of 128");
    auto m = new qpe_mlp();
    try {
      m->ctx = ctx;
      m->n_bits = n_bits;
      m->n_feat = n_feat;
      m->Bp = batch;
      mlp_alloc(m);
      // Uniform(-1/sqrt(fan_in), 1/sqrt(fan_in)) weights from a seeded generator,
      // zero biases; the padded input columns and output rows are zero.
      std::vector<float> p(qpe_mlp::nparams, 0.f);
      uint64_t st = seed ^ 0x243f6a8885a308d3ull;
      auto uni = [&]() {
        st += 0x9e3779b97f4a7c15ull;
        uint64_t z = st;
        z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
        z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
        z ^= z >> 31;
        return (double)(z >> 11) * (1.0 / 9007199254740992.0) * 2.0 - 1.0;
      };
      const uint32_t n_in = n_bits + n_feat;
      for (uint32_t o = 0; o < 256; ++o)
        for (uint32_t i = 0; i < n_in; ++i) p[qpe_mlp::oW1 + o * 64 + i] = (float)(uni() / std::sqrt((double)n_in));
      for (size_t i = 0; i < 256 * 256; ++i) p[qpe_mlp::oW2 + i] = (float)(uni() / 16.0);
      for (size_t i = 0; i < 256 * 256; ++i) p[qpe_mlp::oW3 + i] = (float)(uni() / 16.0);
      for (size_t i = 0; i < 2 * 256; ++i) p[qpe_mlp::oW4 + i] = (float)(uni() / 16.0);
      QPE_CK(cudaMemcpy(m->params.p, p.data(), p.size() * 4, cudaMemcpyHostToDevice));
      cast_all(m, ctx->stream);
      QPE_CK(cudaStreamSynchronize(ctx->stream));
    } catch (...) {
      delete m;
      throw;
    }
    *out = m;
  });
}

int qpe_mlp_destroy(qpe_mlp* m) {
  return guard([&] {
    if (m) {
      use_ctx(m->ctx);
      cudaStreamSynchronize(m->ctx->stream);
    }
    delete m;
  });
}

int qpe_mlp_num_params(const qpe_mlp* m, uint64_t* n) {
  return guard([&] {
    if (!m || !n) throw Error(QPE_ERR_INVALID, "null argument");
    *n = qpe_mlp::nparams;
  });
}

int qpe_mlp_get_params(qpe_mlp* m, float* host) {
  return guard([&] {
    if (!m || !host) throw Error(QPE_ERR_INVALID, "null argument");
    use_ctx(m->ctx);
    QPE_CK(cudaStreamSynchronize(m->ctx->stream));
    QPE_CK(cudaMemcpy(host, m->params.p, qpe_mlp::nparams * 4, cudaMemcpyDeviceToHost));
  });
}

int qpe_mlp_set_params(qpe_mlp* m, const float* host) {
  return guard([&] {
    if (!m || !host) throw Error(QPE_ERR_INVALID, "null argument");
    use_ctx(m->ctx);
    std::vector<float> p(host, host + qpe_mlp::nparams);
    // keep the padding zero: input columns past n_bits + n_feat, output rows past 1
    for (uint32_t o = 0; o < 256; ++o)
      for (uint32_t i = m->n_bits + m->n_feat; i < 64; ++i) p[qpe_mlp::oW1 + o * 64 + i] = 0.f;
    for (size_t i = 2 * 256; i < 16 * 256; ++i) p[qpe_mlp::oW4 + i] = 0.f;
    for (size_t i = 2; i < 16; ++i) p[qpe_mlp::ob4 + i] = 0.f;
    QPE_CK(cudaMemcpy(m->params.p, p.data(), p.size() * 4, cudaMemcpyHostToDevice));
    cast_all(m, m->ctx->stream);
    QPE_CK(cudaStreamSynchronize(m->ctx->stream));
  });
}

int qpe_mlp_set_data(qpe_mlp* m, const uint64_t* bits, const float* log_abs, const float* phase, const float* weight,
                     uint64_t count) {
  return qpe_mlp_set_data2(m, bits, nullptr, log_abs, phase, weight, count);
}

// The model's feature count must be 0 or the caller must give the features.
static void check_feats(const qpe_mlp* m, const float* feats) {
  if (m->n_feat && !feats) throw Error(QPE_ERR_INVALID, "the model takes features: pass them");
}

int qpe_mlp_set_data2(qpe_mlp* m, const uint64_t* bits, const float* feats, const float* log_abs, const float* phase,
                      const float* weight, uint64_t count) {
  return guard([&] {
    if (!m || !bits || !log_abs || !phase || !weight || !count) throw Error(QPE_ERR_INVALID, "null argument");
    check_feats(m, feats);
    use_ctx(m->ctx);
    m->dfeat.alloc(std::max<uint64_t>(1, count * m->n_feat) * 4);
    if (m->n_feat) QPE_CK(cudaMemcpy(m->dfeat.p, feats, count * m->n_feat * 4, cudaMemcpyHostToDevice));
    m->dbits.alloc(count * 8);
    m->dla.alloc(count * 4);
    m->dph.alloc(count * 4);
    m->dw.alloc(count * 4);
    QPE_CK(cudaMemcpy(m->dbits.p, bits, count * 8, cudaMemcpyHostToDevice));
    QPE_CK(cudaMemcpy(m->dla.p, log_abs, count * 4, cudaMemcpyHostToDevice));
    QPE_CK(cudaMemcpy(m->dph.p, phase, count * 4, cudaMemcpyHostToDevice));
    QPE_CK(cudaMemcpy(m->dw.p, weight, count * 4, cudaMemcpyHostToDevice));
    m->nsamples = count;
    if (m->train_exec) cudaGraphExecDestroy(m->train_exec);
    m->train_exec = nullptr;
  });
}

int qpe_mlp_train(qpe_mlp* m, uint32_t steps, float lr, uint64_t seed, float* losses) {
  return guard([&] {
    if (!m) throw Error(QPE_ERR_INVALID, "null model");
    if (!m->nsamples) throw Error(QPE_ERR_INVALID, "no training data (qpe_mlp_set_data)");
    use_ctx(m->ctx);
    cudaStream_t s = m->ctx->stream;
    DevBuf hist;  // per-step losses, copied back once
    hist.alloc((size_t)std::max(steps, 1u) * 4);
    QPE_CK(cudaMemsetAsync(hist.p, 0, hist.bytes, s));
    for (uint32_t t = 0; t < steps; ++t) {
      ++m->adam_t;
      const float c1 = 1.0f / (1.0f - std::pow(0.9f, (float)m->adam_t));
      const float c2 = 1.0f / (1.0f - std::pow(0.999f, (float)m->adam_t));
      k_gather_batch<<<m->Bp, 64, 0, s>>>(m->dbits.as<uint64_t>(), m->dfeat.as<float>(), m->n_feat,
                                           m->dla.as<float>(), m->dph.as<float>(), m->dw.as<float>(), m->nsamples,
                                           m->Bp, m->Bp, m->n_bits, 1, seed,
                                           m->step.as<uint64_t>(), m->X0.as<bf16>(), m->bla.as<float>(),
                                           m->bph.as<float>(), m->bw.as<float>());
      QPE_CK(cudaGetLastError());
      forward(m, s);
      backward(m, m->Bp, s, hist.as<float>() + t);
      adam(m, lr, s, c1, c2);
      k_add_u64<<<1, 1, 0, s>>>(m->step.as<uint64_t>(), 1);
    }
    if (losses) QPE_CK(cudaMemcpyAsync(losses, hist.p, (size_t)steps * 4, cudaMemcpyDeviceToHost, s));
    QPE_CK(cudaStreamSynchronize(s));
    check_err(m);
  });
}

int qpe_mlp_forward(qpe_mlp* m, const uint64_t* bits, uint64_t count, float* out) {
  return qpe_mlp_forward2(m, bits, nullptr, count, out);
}

int qpe_mlp_forward2(qpe_mlp* m, const uint64_t* bits, const float* feats, uint64_t count, float* out) {
  return guard([&] {
    if (!m || (count && (!bits || !out))) throw Error(QPE_ERR_INVALID, "null argument");
    if (count) check_feats(m, feats);
    use_ctx(m->ctx);
    cudaStream_t s = m->ctx->stream;
    DevBuf db, df;
    db.alloc(std::max<uint64_t>(count, 1) * 8);
    QPE_CK(cudaMemcpy(db.p, bits, count * 8, cudaMemcpyHostToDevice));
    df.alloc(std::max<uint64_t>(1, count * m->n_feat) * 4);
    if (m->n_feat && count) QPE_CK(cudaMemcpy(df.p, feats, count * m->n_feat * 4, cudaMemcpyHostToDevice));
    std::vector<float> y((size_t)m->Bp * 16);
    for (uint64_t c0 = 0; c0 < count; c0 += m->Bp) {
      const uint32_t n = (uint32_t)std::min<uint64_t>(m->Bp, count - c0);
      k_gather_batch<<<m->Bp, 64, 0, s>>>(db.as<uint64_t>() + c0, df.as<float>() + c0 * m->n_feat, m->n_feat,
                                           nullptr, nullptr, nullptr, n, n, m->Bp, m->n_bits, 0, 0,
                                           m->step.as<uint64_t>(), m->X0.as<bf16>(), m->bla.as<float>(),
                                           m->bph.as<float>(), m->bw.as<float>());
      QPE_CK(cudaGetLastError());
      forward(m, s);
      QPE_CK(cudaMemcpyAsync(y.data(), m->Y.p, (size_t)n * 16 * 4, cudaMemcpyDeviceToHost, s));
      QPE_CK(cudaStreamSynchronize(s));
      for (uint32_t i = 0; i < n; ++i) {
        out[2 * (c0 + i)] = y[(size_t)i * 16];
        out[2 * (c0 + i) + 1] = y[(size_t)i * 16 + 1];
      }
    }
    check_err(m);
  });
}

int qpe_mlp_gradients(qpe_mlp* m, const uint64_t* bits, const float* log_abs, const float* phase,
                      const float* weight, uint32_t count, float* grads, float* loss) {
  return qpe_mlp_gradients2(m, bits, nullptr, log_abs, phase, weight, count, grads, loss);
}

int qpe_mlp_gradients2(qpe_mlp* m, const uint64_t* bits, const float* feats, const float* log_abs, const float* phase,
                       const float* weight, uint32_t count, float* grads, float* loss) {
  return guard([&] {
    if (!m || !bits || !log_abs || !phase || !weight || !grads) throw Error(QPE_ERR_INVALID, "null argument");
    if (count == 0 || count > m->Bp) throw Error(QPE_ERR_INVALID, "count must be in 1..batch");
    check_feats(m, feats);
    use_ctx(m->ctx);
    cudaStream_t s = m->ctx->stream;
    DevBuf db, dl, dp, dw, df;
    df.alloc(std::max<uint64_t>(1, (uint64_t)count * m->n_feat) * 4);
    if (m->n_feat) QPE_CK(cudaMemcpy(df.p, feats, (size_t)count * m->n_feat * 4, cudaMemcpyHostToDevice));
    db.alloc(count * 8);
    dl.alloc(count * 4);
    dp.alloc(count * 4);
    dw.alloc(count * 4);
    QPE_CK(cudaMemcpy(db.p, bits, count * 8, cudaMemcpyHostToDevice));
    QPE_CK(cudaMemcpy(dl.p, log_abs, count * 4, cudaMemcpyHostToDevice));
    QPE_CK(cudaMemcpy(dp.p, phase, count * 4, cudaMemcpyHostToDevice));
    QPE_CK(cudaMemcpy(dw.p, weight, count * 4, cudaMemcpyHostToDevice));
    QPE_CK(cudaMemsetAsync(m->loss.p, 0, 4, s));
    k_gather_batch<<<m->Bp, 64, 0, s>>>(db.as<uint64_t>(), df.as<float>(), m->n_feat, dl.as<float>(), dp.as<float>(),
                                         dw.as<float>(), count, count, m->Bp, m->n_bits, 0, 0,
                                         m->step.as<uint64_t>(), m->X0.as<bf16>(), m->bla.as<float>(),
                                         m->bph.as<float>(), m->bw.as<float>());
    QPE_CK(cudaGetLastError());
    forward(m, s);
    backward(m, count, s, m->loss.as<float>());
    QPE_CK(cudaMemcpyAsync(grads, m->grads.p, qpe_mlp::nparams * 4, cudaMemcpyDeviceToHost, s));
    if (loss) QPE_CK(cudaMemcpyAsync(loss, m->loss.p, 4, cudaMemcpyDeviceToHost, s));
    QPE_CK(cudaStreamSynchronize(s));
    check_err(m);
  });
}

int qpe_mlp_tensor_flops_per_step(const qpe_mlp* m, double* flops) {
  return guard([&] {
    if (!m || !flops) throw Error(QPE_ERR_INVALID, "null argument");
    *flops = m->tensor_flops_per_step;
  });
}

int qpe_gemm_bf16(qpe_context* ctx, uint32_t M, uint32_t N, uint32_t K, const uint16_t* A, const uint16_t* B,
                  float* D, uint32_t tile_n) {
  return guard([&] {
    use_ctx(ctx);
    if (!A || !B || !D) throw Error(QPE_ERR_INVALID, "null argument");
    if (tile_n != 16 && tile_n != 64 && tile_n != 256) throw Error(QPE_ERR_INVALID, "tile_n must be 16, 64 or 256");
    DevBuf dA, dB, dD, e;
    dA.alloc((size_t)M * K * 2);
    dB.alloc((size_t)N * K * 2);
    dD.alloc((size_t)M * N * 4);
    e.alloc(16);
    QPE_CK(cudaMemset(e.p, 0, 16));
    QPE_CK(cudaMemcpy(dA.p, A, (size_t)M * K * 2, cudaMemcpyHostToDevice));
    QPE_CK(cudaMemcpy(dB.p, B, (size_t)N * K * 2, cudaMemcpyHostToDevice));
    DevBuf scratch;
    const size_t se = (size_t)M * N * 16;
    scratch.alloc(se * 4);
    Gemm G = make_gemm_splitk(tile_n, dA.p, K, dB.p, K, M, N, K, dD.as<float>(), N, scratch.as<float>(), se,
                              (uint32_t)ctx->num_sms, e.as<int>());
    QPE_CK(launch_gemm(G, ctx->stream));
    QPE_CK(cudaStreamSynchronize(ctx->stream));
    int err = 0;
    QPE_CK(cudaMemcpy(&err, e.p, 4, cudaMemcpyDeviceToHost));
    if (err) throw Error(QPE_ERR_TIMEOUT, "tensor-core GEMM: a pipeline wait ran out");
    QPE_CK(cudaMemcpy(D, dD.p, (size_t)M * N * 4, cudaMemcpyDeviceToHost));
  });
}

int qpe_selftest_bounded_wait(qpe_context* ctx, uint32_t max_tries, int arrive) {
  return guard([&] {
    use_ctx(ctx);
    if (max_tries == 0) throw Error(QPE_ERR_INVALID, "max_tries must be positive");
    DevBuf e;
    e.alloc(16);
    QPE_CK(cudaMemsetAsync(e.p, 0, 16, ctx->stream));
    k_wait_probe<<<1, 32, 0, ctx->stream>>>(max_tries, arrive ? 1 : 0, e.as<int>());
    QPE_CK(cudaGetLastError());
    int err = 0;
    QPE_CK(cudaMemcpyAsync(&err, e.p, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
    QPE_CK(cudaStreamSynchronize(ctx->stream));
    if (err)
      throw Error(QPE_ERR_TIMEOUT, "bounded device wait ran out after " + std::to_string(max_tries) +
                                       " polls (mbarrier never completed); the kernel returned and the context is usable");
  });
}

}  // extern "C"
