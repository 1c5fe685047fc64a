// kernels.cu - combinatorial device kernels: colex rank / unrank of fixed-weight
// bit strings, incremental swap ranks, line strings, and the per-term index
// tables (the device form of the discover*_BVs run tables,
// cpp/time_evolution_over_terms.hpp:1160-1411).
#include <cuda_runtime.h>
#include <stdint.h>

#include "kernels.h"

namespace qpe {

// The reference's nChoosek (cpp/util.hpp:49-60), including its unsigned
// wrap-around for large n and its value n for negative k.
static uint64_t ref_nck_host(int n, int k) {
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

void host_ref_binom_table(uint64_t* out) {
  for (int n = 0; n < 64; ++n)
    for (int k = 0; k < BINOM_K; ++k) out[n * BINOM_K + k] = ref_nck_host(n, k);
}

__device__ __forceinline__ uint64_t bn(const uint64_t* __restrict__ t, int n, int k) {
  return __ldg(t + n * BINOM_K + k);
}

// nChoosek for any int k >= -1 (negative k gives n, as the reference does).
__device__ __forceinline__ int64_t ref_nck(const uint64_t* __restrict__ t, int n, int k) {
  if (k < 0) return n;
  if (k >= BINOM_K) return 0;
  return (int64_t)bn(t, n, k);
}

// OffsetComputer::rank (cpp/offset_computer.hpp:16-27): walk the set bits with
// __ffsll; the i-th set bit (1-based order i) at position pos adds C(pos, i).
__device__ __forceinline__ int64_t d_rank(const uint64_t* __restrict__ t, uint64_t bv) {
  int64_t r = 0;
  int order = 1;
  while (bv) {
    const int pos = __ffsll((long long)bv) - 1;
    r += (int64_t)bn(t, pos, order);  // order <= 64 < BINOM_K
    ++order;
    bv &= bv - 1;
  }
  return r;
}

// Colex unrank by one thread: the highest set bit of the rank-r weight-w string
// is the largest p with C(p, w) <= r; repeat for w - 1 below it.
__device__ __forceinline__ uint32_t d_unrank32(const uint64_t* __restrict__ t, uint64_t r, int w, int nbits) {
  uint32_t s = 0;
  int p = nbits - 1;
  for (int k = w; k >= 1; --k) {
    while (p >= k && bn(t, p, k) > r) --p;
    s |= 1u << p;
    r -= bn(t, p, k);
    --p;
  }
  return s;
}

__global__ void k_rank(const uint64_t* __restrict__ tab, const uint64_t* __restrict__ bvs, int64_t* __restrict__ out,
                       size_t n) {
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    out[i] = d_rank(tab, bvs[i]);
}

// Warp-cooperative unrank: for each bit of the result the 32 lanes test one
// candidate position each (C(lane, k) <= r), and a ballot picks the highest lane
// that passes. One warp finishes one rank per `weight` ballots.
__global__ void k_unrank_ballot(const uint64_t* __restrict__ tab, uint32_t nbits, uint32_t weight,
                                const int64_t* __restrict__ ranks, uint64_t* __restrict__ out, size_t n) {
  const uint32_t lane = threadIdx.x & 31;
  const size_t warp = ((size_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const size_t nwarps = ((size_t)gridDim.x * blockDim.x) >> 5;
  for (size_t i = warp; i < n; i += nwarps) {
    uint64_t r = (uint64_t)ranks[i];
    uint32_t s = 0;
    int hi = (int)nbits - 1;
    for (int k = (int)weight; k >= 1; --k) {
      const bool ok = (int)lane <= hi && (int)lane >= k - 1 && bn(tab, lane, k) <= r;
      const unsigned mask = __ballot_sync(0xffffffffu, ok);
      const int p = 31 - __clz(mask);
      s |= 1u << p;
      r -= bn(tab, p, k);
      hi = p - 1;
    }
    if (lane == 0) out[i] = s;
  }
}

__global__ void k_line_strings(const uint64_t* __restrict__ tab, uint32_t nbits, uint32_t weight,
                               uint32_t* __restrict__ out, uint32_t count) {
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < count; i += gridDim.x * blockDim.x)
    out[i] = d_unrank32(tab, i, (int)weight, (int)nbits);
}

// Inserts a zero at each ascending fixed position (the lo / mid / hi segments of
// the discover routines).
__device__ __forceinline__ uint32_t spread(uint32_t free_bits, const uint8_t* fixed, int nfixed) {
  uint32_t out = free_bits;
  for (int i = 0; i < nfixed; ++i) {
    const uint32_t f = fixed[i];
    const uint32_t low = out & ((1u << f) - 1u);
    out = low | ((out >> f) << (f + 1));
  }
  return out;
}

__device__ __forceinline__ uint32_t between_parity(uint32_t full, uint32_t lo, uint32_t hi) {
  if (hi <= lo + 1) return 0;
  const uint32_t mask = ((1u << (hi - lo - 1)) - 1u) << (lo + 1);
  return __popc(full & mask) & 1u;
}

// One thread per table entry. Entry j of a table is the j-th free string in colex
// order, so the table equals the reference's runs expanded in order.
__global__ void k_build_tables(const uint64_t* __restrict__ tab, const AxisTable* __restrict__ tabs,
                               const uint32_t* __restrict__ start, uint32_t ntabs, uint64_t total,
                               uint32_t* __restrict__ pool) {
  for (uint64_t e = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; e < total;
       e += (uint64_t)gridDim.x * blockDim.x) {
    uint32_t lo = 0, hi = ntabs;  // largest t with start[t] <= e
    while (hi - lo > 1) {
      const uint32_t mid = (lo + hi) >> 1;
      if (start[mid] <= e) lo = mid; else hi = mid;
    }
    const AxisTable T = tabs[lo];
    const uint32_t j = (uint32_t)(e - start[lo]);
    uint8_t fx[4] = {T.o[0], T.o[1], T.o[2], T.o[3]};
    // Fixed orbitals of each kind (program.h), sorted ascending.
    int nf = T.nfixed;
    for (int a = 1; a < nf; ++a)
      for (int b = a; b > 0 && fx[b - 1] > fx[b]; --b) {
        const uint8_t x = fx[b];
        fx[b] = fx[b - 1];
        fx[b - 1] = x;
      }
    int nocc = (T.kind == AX_N || T.kind == AX_CA) ? 1 : 2;
    const uint32_t fr = d_unrank32(tab, j, (int)T.weight - nocc, (int)T.nbits - nf);
    const uint32_t base = spread(fr, fx, nf);
    // Orbital slots per kind (program.h): N {q}; NN {p, r}; CA {p, r};
    // CNA {p, q, r}; CCAA {p, q, r, s}.
    switch (T.kind) {
      case AX_N:
        pool[T.offset + j] = (uint32_t)d_rank(tab, base | (1u << T.o[0]));
        break;
      case AX_NN:
        pool[T.offset + j] = (uint32_t)d_rank(tab, base | (1u << T.o[0]) | (1u << T.o[1]));
        break;
      case AX_CA: {  // 01 side r, 10 side p; parity of the bits between them (:1301)
        const uint32_t p = T.o[0], r = T.o[1];
        const uint32_t i01 = (uint32_t)d_rank(tab, base | (1u << r));
        const uint32_t i10 = (uint32_t)d_rank(tab, base | (1u << p));
        const uint32_t par = between_parity(base, min(p, r), max(p, r));
        pool[T.offset + 2 * j] = i01 | (par << 31);
        pool[T.offset + 2 * j + 1] = i10;
        break;
      }
      case AX_CNA: {  // q occupied; 01 side r, 10 side p (:1240-1251)
        const uint32_t p = T.o[0], q = T.o[1], r = T.o[2];
        const uint32_t occ = base | (1u << q);
        const uint32_t i01 = (uint32_t)d_rank(tab, occ | (1u << r));
        const uint32_t i10 = (uint32_t)d_rank(tab, occ | (1u << p));
        // Occupied orbitals strictly between p and r, q included when inside.
        const uint32_t par = between_parity(occ, min(p, r), max(p, r));
        pool[T.offset + 2 * j] = i01 | (par << 31);
        pool[T.offset + 2 * j + 1] = i10;
        break;
      }
      case AX_CCAA: {  // 01 side r, s; 10 side p, q; parity(midlo) + parity(midhi) (:1187)
        const uint32_t p = T.o[0], q = T.o[1], r = T.o[2], s = T.o[3];
        const uint32_t i01 = (uint32_t)d_rank(tab, base | (1u << r) | (1u << s));
        const uint32_t i10 = (uint32_t)d_rank(tab, base | (1u << p) | (1u << q));
        const uint32_t par = between_parity(base, fx[0], fx[1]) ^ between_parity(base, fx[2], fx[3]);
        pool[T.offset + 2 * j] = i01 | (par << 31);
        pool[T.offset + 2 * j + 1] = i10;
        break;
      }
    }
  }
}

// Incremental ranks of OffsetComputer (cpp/offset_computer.hpp:71-192) for one bit
// vector: the prefix tables GEP/GEM (suffix sums from a position up) are built in
// shared memory, then each thread answers queries.
__global__ void k_rank_with_swaps(const uint64_t* __restrict__ tab, uint32_t n, uint64_t bv,
                                  const uint32_t* __restrict__ swaps, int64_t* __restrict__ out, size_t nq) {
  __shared__ int64_t GEP[2][64], GEM[2][64], GTP[2][64], GTM[2][64];
  __shared__ int order[64];
  __shared__ int64_t bv_rank;
  const int i = threadIdx.x;
  if (i < (int)n) order[i] = __popcll(bv & ((2ull << i) - 1ull));
  if (i == 0) bv_rank = d_rank(tab, bv);
  __syncthreads();
  if (i < (int)n) {
    const bool bit = (bv >> i) & 1ull;
    for (int v = 0; v < 2; ++v) {
      GEP[v][i] = bit ? -ref_nck(tab, i, order[i]) + ref_nck(tab, i, order[i] + v + 1) : 0;
      GEM[v][i] = bit ? -ref_nck(tab, i, order[i]) + ref_nck(tab, i, order[i] - (v + 1)) : 0;
    }
  }
  __syncthreads();
  if (i < 2) {  // suffix sums, then the strictly-greater tables
    for (int k = (int)n - 2; k >= 0; --k) {
      GEP[i][k] += GEP[i][k + 1];
      GEM[i][k] += GEM[i][k + 1];
    }
    GTP[i][n - 1] = 0;
    GTM[i][n - 1] = 0;
    for (int k = (int)n - 2; k >= 0; --k) {
      GTP[i][k] = GEP[i][k + 1];
      GTM[i][k] = GEM[i][k + 1];
    }
  }
  __syncthreads();
  auto bit = [&](uint32_t p) -> uint32_t { return (uint32_t)((bv >> p) & 1ull); };
  auto plus = [&](int N, uint32_t lo, uint32_t hi) { return GTP[N - 1][lo] - GEP[N - 1][hi]; };
  auto minus = [&](int N, uint32_t lo, uint32_t hi) { return GTM[N - 1][lo] - GEM[N - 1][hi]; };
  auto destroy = [&](uint32_t b) { return -ref_nck(tab, (int)b, order[b]); };
  auto create = [&](uint32_t b, int o) { return ref_nck(tab, (int)b, o); };
  auto swap1 = [&](uint32_t a, uint32_t b) -> int64_t {
    if (bit(a) == bit(b)) return bv_rank;
    const uint32_t lo = min(a, b), hi = max(a, b);
    if (bit(lo)) return bv_rank + destroy(lo) + create(hi, order[hi]) + minus(1, lo, hi);
    return bv_rank + destroy(hi) + create(lo, order[lo] + 1) + plus(1, lo, hi);
  };
  for (size_t qi = (size_t)blockIdx.x * blockDim.x + threadIdx.x; qi < nq; qi += (size_t)gridDim.x * blockDim.x) {
    const uint32_t a = swaps[4 * qi], b = swaps[4 * qi + 1], c = swaps[4 * qi + 2], d = swaps[4 * qi + 3];
    if (a >= n || b >= n) { out[qi] = -1; continue; }
    if (c == 0xffffffffu) { out[qi] = swap1(a, b); continue; }
    if (c >= n || d >= n) { out[qi] = -1; continue; }
    const uint32_t sum = bit(a) + bit(b) + bit(c) + bit(d);
    if (sum == 0 || sum == 4) { out[qi] = bv_rank; continue; }
    uint32_t pos[4] = {a, b, c, d};
    for (int x = 1; x < 4; ++x)
      for (int y = x; y > 0 && pos[y - 1] > pos[y]; --y) {
        const uint32_t tmp = pos[y];
        pos[y] = pos[y - 1];
        pos[y - 1] = tmp;
      }
    const uint32_t cfg = bit(pos[0]) | (bit(pos[1]) << 1) | (bit(pos[2]) << 2) | (bit(pos[3]) << 3);
    int64_t v;
    if (cfg == 0x3) {
      v = bv_rank + minus(1, pos[0], pos[1]) + minus(2, pos[1], pos[2]) + minus(1, pos[2], pos[3]) +
          destroy(pos[0]) + destroy(pos[1]) + create(pos[2], order[pos[2]] - 1) + create(pos[3], order[pos[3]]);
    } else if (cfg == 0xC) {
      v = bv_rank + plus(1, pos[0], pos[1]) + plus(2, pos[1], pos[2]) + plus(1, pos[2], pos[3]) +
          destroy(pos[2]) + destroy(pos[3]) + create(pos[0], order[pos[0]] + 1) + create(pos[1], order[pos[1]] + 2);
    } else if (cfg == 0x5 || cfg == 0x6 || cfg == 0x9 || cfg == 0xA) {
      v = swap1(a, b) + swap1(c, d) - bv_rank;
    } else {
      out[qi] = -1;
      continue;
    }
    out[qi] = (int64_t)(uint32_t)v;  // the reference keeps this in an unsigned (:160)
  }
}

static uint32_t grid_for(uint64_t n, uint32_t block) {
  uint64_t g = (n + block - 1) / block;
  if (g < 1) g = 1;
  if (g > 65535ull * 16) g = 65535ull * 16;
  return (uint32_t)g;
}

cudaError_t launch_rank(const uint64_t* d_binom, const uint64_t* bvs, int64_t* ranks, size_t n, cudaStream_t s) {
  if (n == 0) return cudaSuccess;
  k_rank<<<grid_for(n, 256), 256, 0, s>>>(d_binom, bvs, ranks, n);
  return cudaGetLastError();
}

cudaError_t launch_unrank(const uint64_t* d_binom, uint32_t nbits, uint32_t weight, const int64_t* ranks,
                          uint64_t* bvs, size_t n, cudaStream_t s) {
  if (n == 0) return cudaSuccess;
  k_unrank_ballot<<<grid_for(n * 32, 256), 256, 0, s>>>(d_binom, nbits, weight, ranks, bvs, n);
  return cudaGetLastError();
}

cudaError_t launch_rank_with_swaps(const uint64_t* d_binom, uint32_t nbits, uint64_t bv, const uint32_t* swaps,
                                   int64_t* out, size_t nq, cudaStream_t s) {
  if (nq == 0) return cudaSuccess;
  uint64_t g = (nq + 127) / 128;
  if (g > 4096) g = 4096;
  k_rank_with_swaps<<<(uint32_t)g, 128, 0, s>>>(d_binom, nbits, bv, swaps, out, nq);
  return cudaGetLastError();
}

cudaError_t launch_line_strings(const uint64_t* d_binom, uint32_t nbits, uint32_t weight, uint32_t* out,
                                uint32_t count, cudaStream_t s) {
  if (count == 0) return cudaSuccess;
  k_line_strings<<<grid_for(count, 256), 256, 0, s>>>(d_binom, nbits, weight, out, count);
  return cudaGetLastError();
}

cudaError_t launch_build_tables(const uint64_t* d_binom, const AxisTable* d_tabs, const uint32_t* d_entry_start,
                                uint32_t ntabs, uint64_t total_entries, uint32_t* d_pool, cudaStream_t s) {
  if (total_entries == 0 || ntabs == 0) return cudaSuccess;
  k_build_tables<<<grid_for(total_entries, 256), 256, 0, s>>>(d_binom, d_tabs, d_entry_start, ntabs, total_entries,
                                                             d_pool);
  return cudaGetLastError();
}

// FP64 FMA throughput probe: kFp64ProbeChains independent FMA chains per
// thread, `iters` steps each, the chains' sum stored so that nothing is dropped.
__global__ void k_fp64_fma_probe(double* __restrict__ out, uint32_t iters) {
  const uint32_t tid = blockIdx.x * blockDim.x + threadIdx.x;
  double a[kFp64ProbeChains];
#pragma unroll
  for (int c = 0; c < kFp64ProbeChains; ++c) a[c] = 1.0 + 1e-9 * (tid + c);
  const double m = 0.999999999, k = 1e-12;
  for (uint32_t i = 0; i < iters; ++i) {
#pragma unroll
    for (int c = 0; c < kFp64ProbeChains; ++c) a[c] = fma(a[c], m, k);
  }
  double s = 0.0;
#pragma unroll
  for (int c = 0; c < kFp64ProbeChains; ++c) s += a[c];
  out[tid] = s;
}

cudaError_t launch_fp64_fma_probe(double* out, uint32_t ctas, uint32_t threads, uint32_t iters, cudaStream_t s) {
  k_fp64_fma_probe<<<ctas, threads, 0, s>>>(out, iters);
  return cudaGetLastError();
}

}  // namespace qpe
