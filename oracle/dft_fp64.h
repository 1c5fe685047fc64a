// dft_fp64.h - FP64 strided forward DFT for the oracle (TEST INFRASTRUCTURE ONLY).
//
// The reference's QIFT calls Intel MKL's DftiComputeForward (cpp/state_vector.hpp:164),
// which is not present in this project. This header is the stand-in: the forward
// transform X_k = sum_j x_j exp(-2 pi i j k / N) (sign -1, as MKL's forward
// transform and cpp/fftw_test.cc:69-71 define it), computed with an iterative
// radix-2 Cooley-Tukey FFT whose twiddles are rounded from long double. Both the
// oracle (oracle/qpe_oracle.cc) and the MKL-DFTI shim used to build the reference
// (oracle/ref_shims/mkl.h) call it, so the oracle and the shimmed reference agree
// bit-for-bit on the QIFT. The QIFT is pinned by definition (the reference's own
// QIFT test, cpp/state_vector.hpp:458-513, expects a bit-reversed peak that a forward
// DFT does not produce).
#ifndef QPE_ORACLE_DFT_FP64_H_
#define QPE_ORACLE_DFT_FP64_H_

#include <cmath>
#include <complex>
#include <cstdint>
#include <vector>

namespace dft_fp64 {

// In-place forward DFT of `howmany` transforms of length N (a power of two):
// transform t holds elements data[t + j * stride], j < N.
inline void forward_strided(std::complex<double>* data, uint64_t N, uint64_t stride, uint64_t howmany) {
  if (N <= 1) return;
  unsigned logn = 0;
  while ((1ull << logn) < N) ++logn;
  std::vector<std::complex<double>> tw(N / 2);
  const long double two_pi = 6.283185307179586476925286766559005768L;
  for (uint64_t k = 0; k < N / 2; ++k) {
    long double ang = -two_pi * (long double)k / (long double)N;
    tw[k] = std::complex<double>((double)cosl(ang), (double)sinl(ang));
  }
  std::vector<uint64_t> rev(N);
  for (uint64_t i = 0; i < N; ++i) {
    uint64_t r = 0;
    for (unsigned b = 0; b < logn; ++b) r |= ((i >> b) & 1ull) << (logn - 1 - b);
    rev[i] = r;
  }
#pragma omp parallel
  {
    std::vector<std::complex<double>> buf(N);
#pragma omp for schedule(static)
    for (int64_t t = 0; t < (int64_t)howmany; ++t) {
      for (uint64_t j = 0; j < N; ++j) buf[rev[j]] = data[(uint64_t)t + j * stride];
      for (uint64_t len = 2; len <= N; len <<= 1) {
        const uint64_t half = len >> 1, step = N / len;
        for (uint64_t base = 0; base < N; base += len)
          for (uint64_t j = 0; j < half; ++j) {
            const std::complex<double> w = tw[j * step];
            const std::complex<double> u = buf[base + j];
            const std::complex<double> v = buf[base + j + half] * w;
            buf[base + j] = u + v;
            buf[base + j + half] = u - v;
          }
      }
      for (uint64_t j = 0; j < N; ++j) data[(uint64_t)t + j * stride] = buf[j];
    }
  }
}

}  // namespace dft_fp64

#endif  // QPE_ORACLE_DFT_FP64_H_
