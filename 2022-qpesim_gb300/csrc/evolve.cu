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
#include <stdint.h>

#include "kernels.h"

namespace qpe {

template <typename R>
struct Cx;
template <>
struct Cx<double> {
  using T = double2;
};
template <>
struct Cx<float> {
  using T = float2;
};

// Arithmetic policies. Exact: separate IEEE roundings (no FMA), the order of
// std::complex<double>'s (ac - bd, ad + bc). Fast: contraction allowed.
struct ExactD {
  static __device__ __forceinline__ double mul(double a, double b) { return __dmul_rn(a, b); }
  static __device__ __forceinline__ double add(double a, double b) { return __dadd_rn(a, b); }
  static __device__ __forceinline__ double sub(double a, double b) { return __dsub_rn(a, b); }
};
template <typename R>
struct Fast {
  static __device__ __forceinline__ R mul(R a, R b) { return a * b; }
  static __device__ __forceinline__ R add(R a, R b) { return a + b; }
  static __device__ __forceinline__ R sub(R a, R b) { return a - b; }
};

template <typename R>
struct Coef4 {
  R e0r, e0i, e1r, e1i, o0r, o0i, o1r, o1i;
  bool reduced;  // m00 real and m01 imaginary for both parities
};

template <typename R>
__device__ __forceinline__ Coef4<R> load_coef(const double* __restrict__ c) {
  Coef4<R> k;
  k.e0r = (R)__ldg(c + 0);
  k.e0i = (R)__ldg(c + 1);
  k.e1r = (R)__ldg(c + 2);
  k.e1i = (R)__ldg(c + 3);
  k.o0r = (R)__ldg(c + 4);
  k.o0i = (R)__ldg(c + 5);
  k.o1r = (R)__ldg(c + 6);
  k.o1i = (R)__ldg(c + 7);
  k.reduced = __ldg(c + 1) == 0.0 && __ldg(c + 2) == 0.0 && __ldg(c + 5) == 0.0 && __ldg(c + 6) == 0.0;
  return k;
}

// Full complex product a * b in the reference's operation order.
template <class A, typename R>
__device__ __forceinline__ void cmul(R ar, R ai, R br, R bi, R& outr, R& outi) {
  outr = A::sub(A::mul(ar, br), A::mul(ai, bi));
  outi = A::add(A::mul(ar, bi), A::mul(ai, br));
}

template <class A, typename C2, typename R>
__device__ __forceinline__ void pair_update(C2& l, C2& r, const Coef4<R>& k, uint32_t par) {
  const R m0r = par ? k.o0r : k.e0r, m0i = par ? k.o0i : k.e0i;
  const R m1r = par ? k.o1r : k.e1r, m1i = par ? k.o1i : k.e1i;
  const C2 vl = l, vr = r;
  if (k.reduced) {
    // m00 = (c, 0), m01 = (0, t): l' = (lx c - ry t, ly c + rx t), r' = (rx c - ly t, lx t + ry c).
    l.x = A::sub(A::mul(vl.x, m0r), A::mul(vr.y, m1i));
    l.y = A::add(A::mul(vl.y, m0r), A::mul(vr.x, m1i));
    r.x = A::sub(A::mul(vr.x, m0r), A::mul(vl.y, m1i));
    r.y = A::add(A::mul(vl.x, m1i), A::mul(vr.y, m0r));
  } else {
    R ar, ai, br, bi;
    cmul<A>(vl.x, vl.y, m0r, m0i, ar, ai);
    cmul<A>(vr.x, vr.y, m1r, m1i, br, bi);
    l.x = A::add(ar, br);
    l.y = A::add(ai, bi);
    cmul<A>(vl.x, vl.y, m1r, m1i, ar, ai);
    cmul<A>(vr.x, vr.y, m0r, m0i, br, bi);
    r.x = A::add(ar, br);
    r.y = A::add(ai, bi);
  }
}

template <class A, typename C2, typename R>
__device__ __forceinline__ void diag_update(C2& v, const Coef4<R>& k) {
  R xr, xi;
  cmul<A>(v.x, v.y, k.e0r, k.e0i, xr, xi);
  v.x = xr;
  v.y = xi;
}

__device__ __forceinline__ bool cond_ok(uint32_t line_str, const DevOp& op) {
  uint32_t m = 0;
  if (op.ncond > 0) m |= 1u << op.cb0;
  if (op.ncond > 1) m |= 1u << op.cb1;
  return (line_str & m) == m;
}

// One pass. PT selects the tile geometry:
//   PASS_COL: tile = W consecutive columns, stage[e * W + w] = block[e][b0 + w]
//   PASS_ROW: tile = one row,               stage[e]         = block[a][e]
//   PASS_MIX: tile = columns (b01, b10),    stage[e * 2 + w] = block[e][w ? b10 : b01]
template <typename R, class A, int PT>
__global__ void k_pass(PassLaunch pl) {
  using C2 = typename Cx<R>::T;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const uint32_t lane = threadIdx.x & 31;
  const uint32_t warp = threadIdx.x >> 5;
  const uint32_t wpc = blockDim.x >> 5;
  const uint32_t Ca = pl.Ca, Cb = pl.Cb;
  const uint32_t W = (PT == PASS_COL) ? pl.W : (PT == PASS_ROW ? 1u : 2u);
  const uint32_t L = (PT == PASS_ROW) ? Cb : Ca;
  const uint32_t logW = __ffs(W) - 1;
  C2* __restrict__ blk = reinterpret_cast<C2*>(pl.work);
  C2* __restrict__ st = reinterpret_cast<C2*>(smem_raw) + (size_t)warp * L * W;
  const uint32_t* __restrict__ pool = pl.pool;
  uint32_t ntiles;
  if (PT == PASS_COL) ntiles = (Cb + W - 1) >> logW;
  else if (PT == PASS_ROW) ntiles = Ca;
  else ntiles = pl.pass.mixcount;

  for (uint32_t tile = blockIdx.x * wpc + warp; tile < ntiles; tile += gridDim.x * wpc) {
    uint32_t b0 = 0, b01 = 0, b10 = 0, parb = 0, row = 0;
    if (PT == PASS_COL) b0 = tile << logW;
    if (PT == PASS_ROW) row = tile;
    if (PT == PASS_MIX) {
      const uint32_t x = __ldg(pool + pl.pass.mixtab + 2 * tile);
      b10 = __ldg(pool + pl.pass.mixtab + 2 * tile + 1);
      b01 = x & 0x7fffffffu;
      parb = x >> 31;
    }
    const uint32_t nl = (PT == PASS_COL) ? min(W, Cb - b0) : W;  // valid lines
    // Line strings for the terms' occupation conditions (at most 32 lines / lane).
    // gather
    for (uint32_t i = lane; i < L * W; i += 32) {
      const uint32_t e = i >> logW, w = i & (W - 1);
      if (w >= nl) continue;
      uint64_t g;
      if (PT == PASS_COL) g = (uint64_t)e * Cb + b0 + w;
      else if (PT == PASS_ROW) g = (uint64_t)row * Cb + e;
      else g = (uint64_t)e * Cb + (w ? b10 : b01);
      st[i] = blk[g];
    }
    __syncwarp();
    for (uint32_t o = pl.pass.op0; o < pl.pass.op1; ++o) {
      const DevOp op = pl.ops[o];
      const Coef4<R> k = load_coef<R>(pl.coef + 8 * (size_t)op.coef);
      if (PT == PASS_MIX) {
        // ABBA: pair (a01 on column b01) <-> (a10 on column b10); parity adds the
        // beta pair's parity (:774).
        for (uint32_t j = lane; j < op.count; j += 32) {
          const uint32_t x = __ldg(pool + op.tab + 2 * j);
          const uint32_t a10 = __ldg(pool + op.tab + 2 * j + 1);
          const uint32_t a01 = x & 0x7fffffffu;
          pair_update<A>(st[a01 * 2 + 0], st[a10 * 2 + 1], k, (x >> 31) ^ parb);
        }
      } else {
        const uint32_t* __restrict__ lstr = (PT == PASS_COL) ? pl.strB : pl.strA;
        const uint32_t line0 = (PT == PASS_COL) ? b0 : row;
        if (op.kind == OPK_PAIR) {
          const uint32_t n = op.count << logW;
          for (uint32_t i = lane; i < n; i += 32) {
            const uint32_t j = i >> logW, w = i & (W - 1);
            if (w >= nl) continue;
            if (op.ncond && !cond_ok(__ldg(lstr + line0 + w), op)) continue;
            const uint32_t x = __ldg(pool + op.tab + 2 * j);
            const uint32_t y = __ldg(pool + op.tab + 2 * j + 1);
            pair_update<A>(st[((x & 0x7fffffffu) << logW) + w], st[(y << logW) + w], k, x >> 31);
          }
        } else if (op.kind == OPK_DIAG_LIST) {
          const uint32_t n = op.count << logW;
          for (uint32_t i = lane; i < n; i += 32) {
            const uint32_t j = i >> logW, w = i & (W - 1);
            if (w >= nl) continue;
            if (op.ncond && !cond_ok(__ldg(lstr + line0 + w), op)) continue;
            const uint32_t e = __ldg(pool + op.tab + j);
            diag_update<A>(st[(e << logW) + w], k);
          }
        } else {  // OPK_DIAG_ALL
          const uint32_t n = L << logW;
          for (uint32_t i = lane; i < n; i += 32) {
            const uint32_t w = i & (W - 1);
            if (w >= nl) continue;
            if (op.ncond && !cond_ok(__ldg(lstr + line0 + w), op)) continue;
            diag_update<A>(st[i], k);
          }
        }
      }
      __syncwarp();
    }
    // scatter
    for (uint32_t i = lane; i < L * W; i += 32) {
      const uint32_t e = i >> logW, w = i & (W - 1);
      if (w >= nl) continue;
      uint64_t g;
      if (PT == PASS_COL) g = (uint64_t)e * Cb + b0 + w;
      else if (PT == PASS_ROW) g = (uint64_t)row * Cb + e;
      else g = (uint64_t)e * Cb + (w ? b10 : b01);
      blk[g] = st[i];
    }
    __syncwarp();
  }
}

size_t pass_stage_elems(const Pass& pass, uint32_t Ca, uint32_t Cb, uint32_t W) {
  if (pass.type == PASS_COL) return (size_t)Ca * W;
  if (pass.type == PASS_ROW) return (size_t)Cb;
  return (size_t)Ca * 2;
}

template <typename R, class A>
static cudaError_t launch_typed(const PassLaunch& pl, cudaStream_t s) {
  using C2 = typename Cx<R>::T;
  const size_t smem = pass_stage_elems(pl.pass, pl.Ca, pl.Cb, pl.W) * sizeof(C2) * pl.warps_per_cta;
  const dim3 block(32 * pl.warps_per_cta);
  switch (pl.pass.type) {
    case PASS_COL: k_pass<R, A, PASS_COL><<<pl.grid, block, smem, s>>>(pl); break;
    case PASS_ROW: k_pass<R, A, PASS_ROW><<<pl.grid, block, smem, s>>>(pl); break;
    default: k_pass<R, A, PASS_MIX><<<pl.grid, block, smem, s>>>(pl); break;
  }
  return cudaGetLastError();
}

cudaError_t launch_pass(const PassLaunch& pl, int dtype, cudaStream_t s) {
  if (dtype == QPE_C128) {
    if (pl.exact) return launch_typed<double, ExactD>(pl, s);
    return launch_typed<double, Fast<double>>(pl, s);
  }
  return launch_typed<float, Fast<float>>(pl, s);
}

template <typename R, class A>
static cudaError_t configure_typed(size_t smem) {
  cudaError_t e;
  if ((e = cudaFuncSetAttribute(k_pass<R, A, PASS_COL>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem)))
    return e;
  if ((e = cudaFuncSetAttribute(k_pass<R, A, PASS_ROW>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem)))
    return e;
  return cudaFuncSetAttribute(k_pass<R, A, PASS_MIX>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
}

cudaError_t configure_pass_kernels(int dtype, size_t smem) {
  if (dtype == QPE_C128) {
    cudaError_t e = configure_typed<double, ExactD>(smem);
    if (e) return e;
    return configure_typed<double, Fast<double>>(smem);
  }
  return configure_typed<float, Fast<float>>(smem);
}

// Snapshot of the working block into block *d_k of the state
// (std::copy_n of :130-132, taken after the power instead of before).
template <typename C2>
__global__ void k_snapshot(const C2* __restrict__ work, C2* __restrict__ state, uint64_t n, const int* d_k) {
  const uint64_t k = (uint64_t)*d_k;
  C2* __restrict__ dst = state + k * n;
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x)
    dst[i] = work[i];
}

__global__ void k_advance(int* d_k) { *d_k += 1; }

cudaError_t launch_snapshot(const void* work, void* state, uint64_t n, const int* d_k, int dtype, cudaStream_t s) {
  uint64_t g = (n + 255) / 256;
  if (g > 152 * 16) g = 152 * 16;
  if (g < 1) g = 1;
  if (dtype == QPE_C128)
    k_snapshot<double2><<<(uint32_t)g, 256, 0, s>>>((const double2*)work, (double2*)state, n, d_k);
  else
    k_snapshot<float2><<<(uint32_t)g, 256, 0, s>>>((const float2*)work, (float2*)state, n, d_k);
  return cudaGetLastError();
}

cudaError_t launch_advance(int* d_k, cudaStream_t s) {
  k_advance<<<1, 1, 0, s>>>(d_k);
  return cudaGetLastError();
}

}  // namespace qpe
