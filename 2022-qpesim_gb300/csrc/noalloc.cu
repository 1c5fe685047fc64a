// noalloc.cu - the QIFT and phase histogram on caller-owned device memory,
// without allocating anything.
//
// Some callers cannot let a library allocate device memory: a host application
// that hands every byte of device memory out of its own pool (a framework's
// caching allocator, a service that sizes its memory once at start-up) and
// forbids libraries from taking more, or a latency-bound loop that cannot afford
// cudaMalloc / cudaFree, which may synchronise the whole device. For them
// qpe_qift_device_noalloc runs the same QIFT kernels as qpe_state_qift on buffers
// the caller passes. The kernels' scratch lives in fixed arrays of this file that
// every GPU which loads the library keeps until the process exits:
//   g_noalloc_scratch  the per-CTA partial rows of the phase histogram
//                      (QPE_NOALLOC_SCRATCH_DOUBLES doubles, 2 MiB plus 8 KiB);
//   g_noalloc_tw64 / g_noalloc_tw32  the twiddle tables of every precision
//                      1..QPE_NOALLOC_MAX_PRECISION in complex128 and complex64
//                      (1,023 values each, 24 KiB together).
//
// Set-up: the first call on a device, with that device current, looks the arrays
// up with cudaGetSymbolAddress, fills the twiddle tables (cudaMemcpyToSymbol, a
// synchronous copy) and raises the QIFT kernel's shared-memory limit to the most
// any precision up to the maximum needs. Make that first call before any stream
// capture. Every later call only launches the QIFT kernel and the histogram
// reduction on the caller's stream. All calls share the partial rows: each call
// writes every partial row it later reads, so nothing has to start at zero, but
// two calls that overlap on the GPU (on different streams, or from different host
// threads) race on them.
#include <cuda_runtime.h>

#include <cmath>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/qpe_gb300.h"
#include "abi_internal.h"
#include "kernels.h"
#include "qpe_common.h"

namespace qpe {

// Partial histogram rows: QPE_NOALLOC_MAX_CTAS rows of 2^QPE_NOALLOC_MAX_PRECISION
// doubles, then 2^QPE_NOALLOC_MAX_PRECISION doubles that earlier versions used for
// the twiddles (kept so that the documented size stays the same).
constexpr uint32_t kNoallocMaxPrecision = QPE_NOALLOC_MAX_PRECISION;
constexpr uint32_t kNoallocMaxCtas = QPE_NOALLOC_MAX_CTAS;
constexpr size_t kNoallocPartialDoubles = (size_t)kNoallocMaxCtas << kNoallocMaxPrecision;
constexpr size_t kNoallocScratchDoubles = kNoallocPartialDoubles + (1u << kNoallocMaxPrecision);
static_assert(kNoallocScratchDoubles == QPE_NOALLOC_SCRATCH_DOUBLES, "scratch size");
// Twiddle tables of precisions 1..max, back to back: precision P's 2^(P-1) values
// start at entry 2^(P-1) - 1.
constexpr uint32_t kNoallocTwiddles = (1u << kNoallocMaxPrecision) - 1;

static __device__ __align__(256) double g_noalloc_scratch[kNoallocScratchDoubles];
static __device__ __align__(256) double2 g_noalloc_tw64[kNoallocTwiddles];
static __device__ __align__(256) float2 g_noalloc_tw32[kNoallocTwiddles];

namespace {
struct NoallocDevice {
  double* scratch = nullptr;
  double2* tw64 = nullptr;
  float2* tw32 = nullptr;
  int num_sms = 0;
};
std::mutex g_noalloc_mu;
NoallocDevice g_noalloc_dev[64];

// Largest dynamic shared memory the QIFT tile takes at any precision: the tile
// width is halved until a tile fits 96 KiB (qpe_state_qift's geometry).
constexpr size_t kNoallocQiftSmem = 96 * 1024;
}  // namespace

// The set-up of `device` (the current device) on its first use; the arrays'
// device addresses afterwards.
static const NoallocDevice& noalloc_device(int device) {
  std::lock_guard<std::mutex> lk(g_noalloc_mu);
  if (device < 0 || device >= 64) throw Error(QPE_ERR_INVALID, "device index out of range");
  NoallocDevice& d = g_noalloc_dev[device];
  if (d.scratch) return d;
  auto ck = [](cudaError_t e, const char* what) {
    if (e != cudaSuccess) throw Error(QPE_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
  };
  void *ps = nullptr, *p64 = nullptr, *p32 = nullptr;
  ck(cudaGetSymbolAddress(&ps, g_noalloc_scratch), "cudaGetSymbolAddress");
  ck(cudaGetSymbolAddress(&p64, g_noalloc_tw64), "cudaGetSymbolAddress");
  ck(cudaGetSymbolAddress(&p32, g_noalloc_tw32), "cudaGetSymbolAddress");
  std::vector<double2> t64(kNoallocTwiddles);
  std::vector<float2> t32(kNoallocTwiddles);
  for (uint32_t P = 1; P <= kNoallocMaxPrecision; ++P) {
    const std::vector<double> tw = twiddle_table(P);
    const uint32_t base = (1u << (P - 1)) - 1;
    for (size_t k = 0; k < tw.size() / 2; ++k) {
      t64[base + k] = make_double2(tw[2 * k], tw[2 * k + 1]);
      t32[base + k] = make_float2((float)tw[2 * k], (float)tw[2 * k + 1]);
    }
  }
  ck(cudaMemcpyToSymbol(g_noalloc_tw64, t64.data(), t64.size() * sizeof(double2)), "twiddle table");
  ck(cudaMemcpyToSymbol(g_noalloc_tw32, t32.data(), t32.size() * sizeof(float2)), "twiddle table");
  ck(configure_qift_kernels(QPE_C128, kNoallocQiftSmem), "QIFT shared-memory limit");
  ck(configure_qift_kernels(QPE_C64, kNoallocQiftSmem), "QIFT shared-memory limit");
  ck(cudaDeviceGetAttribute(&d.num_sms, cudaDevAttrMultiProcessorCount, device), "cudaDeviceGetAttribute");
  d.tw64 = static_cast<double2*>(p64);
  d.tw32 = static_cast<float2*>(p32);
  d.scratch = static_cast<double*>(ps);  // set last: marks the set-up done
  return d;
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
    const NoallocDevice& d = noalloc_device(device);
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    const uint32_t N = 1u << precision;
    const size_t esz = dtype == QPE_C128 ? 16 : 8;
    // The same tile geometry as qpe_state_qift.
    uint32_t T = 32;
    while (T > 1 && ((size_t)N * esz * T > kNoallocQiftSmem || T > ld)) T >>= 1;
    uint64_t tiles = (ld + T - 1) / T;
    uint64_t grid = (uint64_t)d.num_sms * 2;
    if (grid > tiles) grid = tiles;
    if (grid > kNoallocMaxCtas) grid = kNoallocMaxCtas;
    const uint32_t base = (1u << (precision - 1)) - 1;
    const void* tw = dtype == QPE_C128 ? static_cast<const void*>(d.tw64 + base) : static_cast<const void*>(d.tw32 + base);
    e = launch_qift(d_state, ld, precision, tw, std::sqrt((double)N), d.scratch, (uint32_t)grid, T, dtype, s);
    if (e == cudaSuccess) e = launch_reduce_partials(d.scratch, (uint32_t)grid, N, d_probs, s);
    if (e != cudaSuccess) throw Error(QPE_ERR_CUDA, cudaGetErrorString(e));
  });
}
