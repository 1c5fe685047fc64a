// mkl.h - stand-in for the subset of Intel MKL DFTI that StateVector::qift uses
// (cpp/state_vector.hpp:133-168). MKL is not part of this project; the transform is
// the oracle's FP64 forward DFT (oracle/dft_fp64.h), sign -1 as MKL's
// DftiComputeForward. TEST INFRASTRUCTURE ONLY.
#ifndef QPE_REF_SHIM_MKL_H_
#define QPE_REF_SHIM_MKL_H_

#include <complex>
#include <cstdarg>
#include <cstdint>

#include "../dft_fp64.h"

typedef long MKL_LONG;

enum DFTI_CONFIG_PARAM {
  DFTI_PLACEMENT = 1,
  DFTI_THREAD_LIMIT,
  DFTI_COMPLEX_STORAGE,
  DFTI_NUMBER_OF_TRANSFORMS,
  DFTI_INPUT_DISTANCE,
  DFTI_OUTPUT_DISTANCE,
  DFTI_INPUT_STRIDES,
  DFTI_OUTPUT_STRIDES,
  DFTI_FORWARD_DOMAIN
};
enum DFTI_CONFIG_VALUE { DFTI_DOUBLE = 100, DFTI_COMPLEX, DFTI_INPLACE, DFTI_COMPLEX_COMPLEX };
#define DFTI_NO_ERROR 0L

struct DFTI_DESCRIPTOR {
  MKL_LONG length = 0;
  MKL_LONG howmany = 1;
  MKL_LONG distance = 1;
  MKL_LONG offset = 0;
  MKL_LONG stride = 1;
};
typedef DFTI_DESCRIPTOR* DFTI_DESCRIPTOR_HANDLE;

inline MKL_LONG DftiCreateDescriptor(DFTI_DESCRIPTOR_HANDLE* h, DFTI_CONFIG_VALUE, DFTI_CONFIG_VALUE, MKL_LONG dim,
                                     ...) {
  if (dim != 1) return 1;
  va_list ap;
  va_start(ap, dim);
  MKL_LONG n = va_arg(ap, MKL_LONG);
  va_end(ap);
  *h = new DFTI_DESCRIPTOR();
  (*h)->length = n;
  return DFTI_NO_ERROR;
}

inline MKL_LONG DftiSetValue(DFTI_DESCRIPTOR_HANDLE h, DFTI_CONFIG_PARAM p, ...) {
  va_list ap;
  va_start(ap, p);
  switch (p) {
    case DFTI_NUMBER_OF_TRANSFORMS: h->howmany = va_arg(ap, MKL_LONG); break;
    case DFTI_INPUT_DISTANCE: h->distance = va_arg(ap, MKL_LONG); break;
    case DFTI_OUTPUT_DISTANCE: (void)va_arg(ap, MKL_LONG); break;
    case DFTI_INPUT_STRIDES: {
      MKL_LONG* s = va_arg(ap, MKL_LONG*);
      h->offset = s[0];
      h->stride = s[1];
      break;
    }
    default: break;
  }
  va_end(ap);
  return DFTI_NO_ERROR;
}

inline MKL_LONG DftiCommitDescriptor(DFTI_DESCRIPTOR_HANDLE) { return DFTI_NO_ERROR; }

inline MKL_LONG DftiComputeForward(DFTI_DESCRIPTOR_HANDLE h, void* data) {
  if (h->distance != 1) return 1;
  auto* x = reinterpret_cast<std::complex<double>*>(data) + h->offset;
  dft_fp64::forward_strided(x, (uint64_t)h->length, (uint64_t)h->stride, (uint64_t)h->howmany);
  return DFTI_NO_ERROR;
}

inline MKL_LONG DftiFreeDescriptor(DFTI_DESCRIPTOR_HANDLE* h) {
  delete *h;
  *h = nullptr;
  return DFTI_NO_ERROR;
}

#endif  // QPE_REF_SHIM_MKL_H_
