// noalloc.cu - the QIFT and phase histogram on caller-owned device memory,
// without allocating anything.
//
// Some callers cannot allocate device memory at the moment they need the QIFT:
// code running while its stream is being captured into a CUDA graph (cudaMalloc
// is not allowed during capture), or a host that hands every byte of device
// memory out of its own pool and forbids a library from taking more. For them
// qpe_qift_device_noalloc runs the same QIFT kernel as qpe_state_qift on buffers
// the caller passes, with the kernel's scratch - the per-CTA partial rows of the
// phase histogram and the twiddle table - in a fixed array of this file
// (QPE_NOALLOC_SCRATCH_DOUBLES doubles, 2 MiB plus 8 KiB) that every GPU which
// loads the library keeps until the process exits.
//
// Set-up: the first call on a device, with that device current, looks the array
// up with cudaGetSymbolAddress and keeps the address; make that first call before
// any stream capture. Every call shares the array: each call writes every partial
// row it later reads, so nothing has to start at zero, but two calls that overlap
// on the GPU (on different streams, or from different host threads) race on it.
#include <cuda_runtime.h>

#include <cmath>
#include <mutex>
#include <string>

#include "../../include/qpe_gb300.h"
#include "kernels.h"
#include "qpe_common.h"

namespace qpe {

// Partial histogram rows: QPE_NOALLOC_MAX_CTAS rows of 2^QPE_NOALLOC_MAX_PRECISION
// doubles, then the twiddle table (2^(P-1) complex values).
constexpr uint32_t kNoallocMaxPrecision = QPE_NOALLOC_MAX_PRECISION;
constexpr uint32_t kNoallocMaxCtas = QPE_NOALLOC_MAX_CTAS;
constexpr size_t kNoallocPartialDoubles = (size_t)kNoallocMaxCtas << kNoallocMaxPrecision;
constexpr size_t kNoallocScratchDoubles = kNoallocPartialDoubles + (1u << kNoallocMaxPrecision);
static_assert(kNoallocScratchDoubles == QPE_NOALLOC_SCRATCH_DOUBLES, "scratch size");

static __device__ __align__(256) double g_noalloc_scratch[kNoallocScratchDoubles];

namespace {
std::mutex g_noalloc_mu;
double* g_noalloc_ptr[64] = {};
}  // namespace

// Device address of the scratch array on the current device (set-up on first use).
static double* noalloc_scratch(int device) {
  std::lock_guard<std::mutex> lk(g_noalloc_mu);
  if (device < 0 || device >= 64) throw Error(QPE_ERR_INVALID, "device index out of range");
  if (!g_noalloc_ptr[device]) {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess) throw Error(QPE_ERR_CUDA, std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));
    g_noalloc_ptr[device] = static_cast<double*>(p);
  }
  return g_noalloc_ptr[device];
}

}  // namespace qpe

using namespace qpe;

extern "C" int qpe_qift_device_noalloc(void* stream, uint32_t precision, uint64_t ld, int dtype, void* d_state,
                                       double* d_probs) {
  return guard([&] {
    if (!d_state || !d_probs) throw Error(QPE_ERR_INVALID, "null device buffer");
    if (dtype != QPE_C128 && dtype != QPE_C64) throw Error(QPE_ERR_INVALID, "unknown dtype");
    if (precision == 0 || precision > kNoallocMaxPrecision)
      throw Error(QPE_ERR_UNSUPPORTED, "qpe_qift_device_noalloc handles precision 1.." +
                                           std::to_string(kNoallocMaxPrecision) + " (fixed scratch size)");
    if (ld == 0) throw Error(QPE_ERR_INVALID, "ld must be positive");
    int device = 0;
    cudaError_t e = cudaGetDevice(&device);
    if (e != cudaSuccess) throw Error(QPE_ERR_NO_DEVICE, std::string("cudaGetDevice: ") + cudaGetErrorString(e));
    double* scratch = noalloc_scratch(device);
    int num_sms = 0;
    e = cudaDeviceGetAttribute(&num_sms, cudaDevAttrMultiProcessorCount, device);
    if (e != cudaSuccess) throw Error(QPE_ERR_CUDA, cudaGetErrorString(e));
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    const uint32_t N = 1u << precision;
    const size_t esz = dtype == QPE_C128 ? 16 : 8;
    // The same tile geometry as qpe_state_qift.
    uint32_t T = 32;
    while (T > 1 && ((size_t)N * esz * T > 96 * 1024 || T > ld)) T >>= 1;
    uint64_t tiles = (ld + T - 1) / T;
    uint64_t grid = (uint64_t)num_sms * 2;
    if (grid > tiles) grid = tiles;
    if (grid > kNoallocMaxCtas) grid = kNoallocMaxCtas;
    // Twiddles exp(-2 pi i k / N), k < N / 2, rounded from long double, copied into
    // the scratch array behind the partial rows.
    double tw[1u << kNoallocMaxPrecision];
    const uint32_t nh = N / 2 ? N / 2 : 1;
    const long double two_pi = 6.283185307179586476925286766559005768L;
    for (uint32_t k = 0; k < nh; ++k) {
      long double ang = -two_pi * (long double)k / (long double)N;
      tw[2 * k] = (double)cosl(ang);
      tw[2 * k + 1] = (double)sinl(ang);
    }
    double* d_tw = scratch + kNoallocPartialDoubles;
    if (dtype == QPE_C128) {
      e = cudaMemcpyAsync(d_tw, tw, 2 * nh * sizeof(double), cudaMemcpyHostToDevice, s);
    } else {
      float twf[1u << kNoallocMaxPrecision];
      for (uint32_t i = 0; i < 2 * nh; ++i) twf[i] = (float)tw[i];
      e = cudaMemcpyAsync(d_tw, twf, 2 * nh * sizeof(float), cudaMemcpyHostToDevice, s);
    }
    if (e != cudaSuccess) throw Error(QPE_ERR_CUDA, std::string("twiddle copy: ") + cudaGetErrorString(e));
    e = configure_qift_kernels(dtype, qift_smem_bytes(precision, T, dtype));
    if (e != cudaSuccess) throw Error(QPE_ERR_CUDA, cudaGetErrorString(e));
    e = launch_qift(d_state, ld, precision, d_tw, std::sqrt((double)N), scratch, (uint32_t)grid, T, dtype, s);
    if (e == cudaSuccess) e = launch_reduce_partials(scratch, (uint32_t)grid, N, d_probs, s);
    if (e != cudaSuccess) throw Error(QPE_ERR_CUDA, cudaGetErrorString(e));
  });
}
