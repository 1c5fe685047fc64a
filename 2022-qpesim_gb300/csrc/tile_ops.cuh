// tile_ops.cuh - the per-tile term application shared by the evolution kernels.
//
// A tile is W lines of one pass (program.h). Lane l of the warp owns line
// l % W for the whole tile and walks the entries j = l / W, l / W + 32 / W, ... of
// every term's index table, so each lane keeps its line's constants (column,
// beta-pair columns, occupation string) in registers. The pair update is the
// reference's updateStateVector (cpp/time_evolution_over_terms.hpp:565-589):
// l' = l*m00 + r*m01, r' = l*m01 + r*m00. In exact mode every product and sum of
// the complex128 arithmetic is rounded separately, in the order of
// std::complex<double>'s (ac - bd, ad + bc), so results are bit-identical to the
// reference built without floating-point contraction; terms whose m00 is real and
// m01 imaginary (every pq / pqqr / pqrs term of the Hamiltonian getters) skip the
// products with exact zeros, which changes no bit.
#ifndef QPE_TILE_OPS_CUH_
#define QPE_TILE_OPS_CUH_

#include <cuda_runtime.h>
#include <stdint.h>

#include "program.h"

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
  const double2 a = __ldg(reinterpret_cast<const double2*>(c));
  const double2 b = __ldg(reinterpret_cast<const double2*>(c) + 1);
  const double2 d = __ldg(reinterpret_cast<const double2*>(c) + 2);
  const double2 e = __ldg(reinterpret_cast<const double2*>(c) + 3);
  k.e0r = (R)a.x; k.e0i = (R)a.y; k.e1r = (R)b.x; k.e1i = (R)b.y;
  k.o0r = (R)d.x; k.o0i = (R)d.y; k.o1r = (R)e.x; k.o1i = (R)e.y;
  k.reduced = a.y == 0.0 && b.x == 0.0 && d.y == 0.0 && e.x == 0.0;
  return k;
}

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
  C2 nl, nr;
  if (k.reduced) {
    // m00 = (c, 0), m01 = (0, t): l' = (lx c - ry t, ly c + rx t), r' = (rx c - ly t, lx t + ry c).
    nl.x = A::sub(A::mul(vl.x, m0r), A::mul(vr.y, m1i));
    nl.y = A::add(A::mul(vl.y, m0r), A::mul(vr.x, m1i));
    nr.x = A::sub(A::mul(vr.x, m0r), A::mul(vl.y, m1i));
    nr.y = A::add(A::mul(vl.x, m1i), A::mul(vr.y, m0r));
  } else {
    R ar, ai, br, bi;
    cmul<A>(vl.x, vl.y, m0r, m0i, ar, ai);
    cmul<A>(vr.x, vr.y, m1r, m1i, br, bi);
    nl.x = A::add(ar, br);
    nl.y = A::add(ai, bi);
    cmul<A>(vl.x, vl.y, m1r, m1i, ar, ai);
    cmul<A>(vr.x, vr.y, m0r, m0i, br, bi);
    nr.x = A::add(ar, br);
    nr.y = A::add(ai, bi);
  }
  l = nl;
  r = nr;
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

// Runs the terms [op0, op1) of a COL or ROW pass on this lane's line. `elem(e)`
// returns a reference to entry e of the line; `active` is false for lanes past
// the last line; `lstr` is the line's occupation string (for conditions).
// The loop is software-pipelined: the next term's descriptor, coefficients and
// this lane's first table entry are loaded while the current term computes, so
// the chain of dependent terms pays the shared-memory latency, not the latency
// of the metadata loads.
template <typename R, class A, class Elem>
__device__ __forceinline__ void run_line_ops(const DevOp* __restrict__ ops, const double* __restrict__ coef,
                                             const uint32_t* __restrict__ pool, uint32_t op0, uint32_t op1,
                                             uint32_t L, uint32_t jl, uint32_t jstep, bool active, uint32_t lstr,
                                             Elem elem) {
  if (op0 >= op1) return;
  auto first_of = [&](const DevOp& d) -> uint2 {
    return (d.kind == OPK_PAIR && jl < d.count) ? __ldg(reinterpret_cast<const uint2*>(pool + d.tab) + jl)
                                                : make_uint2(0u, 0u);
  };
  DevOp op = ops[op0];
  Coef4<R> k = load_coef<R>(coef + 8 * (size_t)op.coef);
  uint2 first = first_of(op);
  for (uint32_t o = op0; o < op1; ++o) {
    DevOp opn = op;
    Coef4<R> kn = k;
    uint2 firstn = make_uint2(0u, 0u);
    if (o + 1 < op1) {
      opn = ops[o + 1];
      kn = load_coef<R>(coef + 8 * (size_t)opn.coef);
      firstn = first_of(opn);
    }
    if (active && (op.ncond == 0 || cond_ok(lstr, op))) {
      if (op.kind == OPK_PAIR) {
        const uint2* __restrict__ t = reinterpret_cast<const uint2*>(pool + op.tab);
        uint2 x = first;
        for (uint32_t j = jl; j < op.count; j += jstep) {
          const uint32_t jn = j + jstep;
          const uint2 xn = jn < op.count ? __ldg(t + jn) : make_uint2(0u, 0u);
          pair_update<A>(elem(x.x & 0x7fffffffu), elem(x.y), k, x.x >> 31);
          x = xn;
        }
      } else if (op.kind == OPK_DIAG_LIST) {
        for (uint32_t j = jl; j < op.count; j += jstep) diag_update<A>(elem(__ldg(pool + op.tab + j)), k);
      } else {
        for (uint32_t e = jl; e < L; e += jstep) diag_update<A>(elem(e), k);
      }
    }
    __syncwarp();
    op = opn;
    k = kn;
    first = firstn;
  }
}

// Runs the pqrs ABBA terms [op0, op1) of a MIX pass on this lane's column pair:
// entry (a01 | par, a10) pairs left(a01) with right(a10), parity adding the beta
// pair's parity parb (cpp/time_evolution_over_terms.hpp:774). Pipelined as
// run_line_ops.
template <typename R, class A, class Left, class Right>
__device__ __forceinline__ void run_mix_ops(const DevOp* __restrict__ ops, const double* __restrict__ coef,
                                            const uint32_t* __restrict__ pool, uint32_t op0, uint32_t op1,
                                            uint32_t jl, uint32_t jstep, bool active, uint32_t parb, Left left,
                                            Right right) {
  if (op0 >= op1) return;
  auto first_of = [&](const DevOp& d) -> uint2 {
    return jl < d.count ? __ldg(reinterpret_cast<const uint2*>(pool + d.tab) + jl) : make_uint2(0u, 0u);
  };
  DevOp op = ops[op0];
  Coef4<R> k = load_coef<R>(coef + 8 * (size_t)op.coef);
  uint2 first = first_of(op);
  for (uint32_t o = op0; o < op1; ++o) {
    DevOp opn = op;
    Coef4<R> kn = k;
    uint2 firstn = make_uint2(0u, 0u);
    if (o + 1 < op1) {
      opn = ops[o + 1];
      kn = load_coef<R>(coef + 8 * (size_t)opn.coef);
      firstn = first_of(opn);
    }
    const uint2* __restrict__ t = reinterpret_cast<const uint2*>(pool + op.tab);
    uint2 x = first;
    if (active) {
      for (uint32_t j = jl; j < op.count; j += jstep) {
        const uint32_t jn = j + jstep;
        const uint2 xn = jn < op.count ? __ldg(t + jn) : make_uint2(0u, 0u);
        pair_update<A>(left(x.x & 0x7fffffffu), right(x.y), k, (x.x >> 31) ^ parb);
        x = xn;
      }
    }
    __syncwarp();
    op = opn;
    k = kn;
    first = firstn;
  }
}

}  // namespace qpe

#endif  // QPE_TILE_OPS_CUH_
