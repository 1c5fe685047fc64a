// qift.cu - the QIFT and the phase histogram.
//
// StateVector::qift (cpp/state_vector.hpp:115-179) is an in-place forward DFT
// (sign -1) of length N = 2^P along the ancilla axis, stride ld = Ca * Cb, for all
// ld columns, followed by division by sqrt(N). Here one CTA owns a tile of T
// consecutive columns: it loads the N x T tile into shared memory in bit-reversed
// row order (coalesced along the columns), runs the radix-2 decimation-in-time
// stages, divides by sqrt(N), writes the tile back and accumulates the per-row
// probabilities |x|^2 of its columns (IdentifyPhaseAmplitudes, :341-372) into a
// per-CTA partial row that a second kernel reduces in a fixed order.
//
// Stages of radix 2^k: the first five stages (spans 2..32) of each column run in
// registers of one warp, lanes exchanging partners with __shfl_xor_sync, so each
// warp finishes a radix-32 block without touching shared memory; the remaining
// stages use shared memory with a barrier per stage.
//
// Complex128 uses separately rounded products and sums in the order of
// std::complex<double> arithmetic and the same long-double-rounded twiddles as the
// oracle's radix-2 FFT, so the transform is reproducible bit for bit.
#include <cuda_runtime.h>

#include <map>
#include <mutex>
#include <stdint.h>

#include "kernels.h"

namespace qpe {

template <typename R>
struct QCx;
template <>
struct QCx<double> {
  using T = double2;
  static __device__ __forceinline__ double mul(double a, double b) { return __dmul_rn(a, b); }
  static __device__ __forceinline__ double add(double a, double b) { return __dadd_rn(a, b); }
  static __device__ __forceinline__ double sub(double a, double b) { return __dsub_rn(a, b); }
};
template <>
struct QCx<float> {
  using T = float2;
  static __device__ __forceinline__ float mul(float a, float b) { return a * b; }
  static __device__ __forceinline__ float add(float a, float b) { return a + b; }
  static __device__ __forceinline__ float sub(float a, float b) { return a - b; }
};

// u, v <- u + v*w, u - v*w (one radix-2 butterfly).
template <typename R, typename C2>
__device__ __forceinline__ void butterfly(C2& u, C2& v, const C2 w) {
  using Q = QCx<R>;
  const R tr = Q::sub(Q::mul(v.x, w.x), Q::mul(v.y, w.y));
  const R ti = Q::add(Q::mul(v.x, w.y), Q::mul(v.y, w.x));
  const C2 a = u;
  u.x = Q::add(a.x, tr);
  u.y = Q::add(a.y, ti);
  v.x = Q::sub(a.x, tr);
  v.y = Q::sub(a.y, ti);
}

template <typename R, typename C2>
__device__ __forceinline__ C2 shfl_xor_c(const C2 v, int m) {
  C2 o;
  o.x = __shfl_xor_sync(0xffffffffu, v.x, m);
  o.y = __shfl_xor_sync(0xffffffffu, v.y, m);
  return o;
}

template <typename R>
__global__ void k_qift(typename QCx<R>::T* __restrict__ state, uint64_t ld, uint32_t P,
                       const typename QCx<R>::T* __restrict__ tw, R norm, double* __restrict__ partial,
                       uint32_t T) {
  using C2 = typename QCx<R>::T;
  using Q = QCx<R>;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  C2* __restrict__ buf = reinterpret_cast<C2*>(smem_raw);  // [N][T]
  const uint32_t N = 1u << P;
  const uint32_t tid = threadIdx.x, nt = blockDim.x;
  const uint64_t ntiles = (ld + T - 1) / T;
  // Per-thread accumulators of the rows this thread reduces (rows tid, tid + nt, ...).
  double acc[8];
#pragma unroll
  for (int i = 0; i < 8; ++i) acc[i] = 0.0;

  for (uint64_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
    const uint64_t c0 = tile * T;
    const uint32_t tw_ = (uint32_t)min((uint64_t)T, ld - c0);
    // Load in bit-reversed row order.
    for (uint32_t i = tid; i < N * T; i += nt) {
      const uint32_t k = i / T, t = i - k * T;
      const uint32_t rk = P ? (__brev(k) >> (32 - P)) : 0;
      C2 v;
      if (t < tw_) v = state[(uint64_t)k * ld + c0 + t];
      else { v.x = 0; v.y = 0; }
      buf[rk * T + t] = v;
    }
    __syncthreads();
    // Spans 2..min(N, 32): butterflies within aligned groups of 32 rows, done by
    // one warp per (group, column) with the 32 rows in its lanes.
    const uint32_t s_reg = P < 5 ? P : 5;
    if (s_reg > 0) {
      const uint32_t G = 1u << s_reg;            // rows per group
      const uint32_t lanes_used = G;             // one row per lane
      const uint32_t warps = nt >> 5;
      const uint32_t warp = tid >> 5, lane = tid & 31;
      const uint32_t jobs = (N / G) * T;         // (group, column) pairs
      for (uint32_t job = warp; job < jobs; job += warps) {
        const uint32_t grp = job / T, t = job - grp * T;
        const uint32_t row = grp * G + (lane & (G - 1));
        C2 x = buf[row * T + t];
        for (uint32_t s = 1; s <= s_reg; ++s) {
          const uint32_t half = 1u << (s - 1);
          const uint32_t j = lane & (half - 1);               // position in the half span
          const C2 w = tw[j * (N >> s)];
          const C2 y = shfl_xor_c<R>(x, (int)half);
          // lower member holds u, upper holds v; both compute the same butterfly
          const bool upper = lane & half;
          C2 u = upper ? y : x, v = upper ? x : y;
          butterfly<R>(u, v, w);
          x = upper ? v : u;
        }
        if (lane < lanes_used) buf[row * T + t] = x;
      }
      __syncthreads();
    }
    // Remaining spans in shared memory.
    for (uint32_t s = s_reg + 1; s <= P; ++s) {
      const uint32_t len = 1u << s, half = len >> 1, step = N >> s;
      for (uint32_t b = tid; b < (N / 2) * T; b += nt) {
        const uint32_t bf = b / T, t = b - bf * T;
        const uint32_t grp = bf / half, j = bf - grp * half;
        const uint32_t i0 = grp * len + j, i1 = i0 + half;
        C2 u = buf[i0 * T + t], v = buf[i1 * T + t];
        butterfly<R>(u, v, tw[j * step]);
        buf[i0 * T + t] = u;
        buf[i1 * T + t] = v;
      }
      __syncthreads();
    }
    // Divide by sqrt(N) (:172-178) and write back.
    for (uint32_t i = tid; i < N * T; i += nt) {
      const uint32_t k = i / T, t = i - k * T;
      if (t >= tw_) continue;
      C2 v = buf[i];
      v.x = v.x / norm;
      v.y = v.y / norm;
      buf[i] = v;
      state[(uint64_t)k * ld + c0 + t] = v;
    }
    __syncthreads();
    // Row probabilities of this tile.
    for (uint32_t k = tid, slot = 0; k < N; k += nt, ++slot) {
      double s = 0.0;
      for (uint32_t t = 0; t < tw_; ++t) {
        const C2 v = buf[k * T + t];
        s += (double)v.x * (double)v.x + (double)v.y * (double)v.y;
      }
      if (slot < 8) acc[slot] += s;
    }
    __syncthreads();
  }
  for (uint32_t k = tid, slot = 0; k < N && slot < 8; k += nt, ++slot) partial[(uint64_t)blockIdx.x * N + k] = acc[slot];
}

size_t qift_smem_bytes(uint32_t P, uint32_t T, int dtype) {
  return (size_t)(1u << P) * T * (dtype == QPE_C128 ? sizeof(double2) : sizeof(float2));
}

// Only ever raises the limit (per device and type), so that registers of
// different sizes can be transformed in any order.
cudaError_t configure_qift_kernels(int dtype, size_t smem) {
  static std::mutex mu;
  static std::map<std::pair<int, int>, size_t> granted;  // (device, dtype) -> bytes
  int dev = 0;
  cudaGetDevice(&dev);
  std::lock_guard<std::mutex> lock(mu);
  size_t& g = granted[{dev, dtype}];
  if (smem <= g) return cudaSuccess;
  const cudaError_t e =
      dtype == QPE_C128 ? cudaFuncSetAttribute(k_qift<double>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem)
                        : cudaFuncSetAttribute(k_qift<float>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e == cudaSuccess) g = smem;
  return e;
}

cudaError_t launch_qift(void* state, uint64_t ld, uint32_t P, const void* tw, double norm, double* partial,
                        uint32_t grid, uint32_t T, int dtype, cudaStream_t s) {
  const size_t smem = qift_smem_bytes(P, T, dtype);
  const uint32_t N = 1u << P;
  uint32_t block = N >= 1024 ? 1024 : (N * T >= 256 ? 256 : 128);
  if (block < N / 8) block = 1024;  // each thread keeps at most 8 row accumulators
  if (dtype == QPE_C128)
    k_qift<double><<<grid, block, smem, s>>>((double2*)state, ld, P, (const double2*)tw, norm, partial, T);
  else
    k_qift<float><<<grid, block, smem, s>>>((float2*)state, ld, P, (const float2*)tw, (float)norm, partial, T);
  return cudaGetLastError();
}

// probs[k] = sum over CTAs of partial[cta][k], in CTA order.
__global__ void k_reduce_partials(const double* __restrict__ partial, uint32_t nparts, uint32_t N,
                                  double* __restrict__ out) {
  for (uint32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < N; k += gridDim.x * blockDim.x) {
    double s = 0.0;
    for (uint32_t p = 0; p < nparts; ++p) s += partial[(uint64_t)p * N + k];
    out[k] = s;
  }
}

cudaError_t launch_reduce_partials(const double* partial, uint32_t nparts, uint32_t N, double* out, cudaStream_t s) {
  k_reduce_partials<<<(N + 255) / 256, 256, 0, s>>>(partial, nparts, N, out);
  return cudaGetLastError();
}

// out[k] = sum over the ld amplitudes of block k of |a|^2, FP64 accumulation, one
// CTA per block, fixed reduction tree.
template <typename C2>
__global__ void k_block_sums(const C2* __restrict__ state, uint64_t ld, double* __restrict__ out) {
  __shared__ double red[32];
  const uint64_t k = blockIdx.x;
  const C2* __restrict__ b = state + k * ld;
  double s = 0.0;
  for (uint64_t i = threadIdx.x; i < ld; i += blockDim.x) {
    const C2 v = b[i];
    s += (double)v.x * (double)v.x + (double)v.y * (double)v.y;
  }
  for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x < 32) {
    s = threadIdx.x < (blockDim.x >> 5) ? red[threadIdx.x] : 0.0;
    for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
    if (threadIdx.x == 0) out[k] = s;
  }
}

cudaError_t launch_block_sums(const void* state, uint64_t ld, uint32_t N, double* out, int dtype, cudaStream_t s) {
  if (dtype == QPE_C128)
    k_block_sums<double2><<<N, 512, 0, s>>>((const double2*)state, ld, out);
  else
    k_block_sums<float2><<<N, 512, 0, s>>>((const float2*)state, ld, out);
  return cudaGetLastError();
}

}  // namespace qpe
