// abi_internal.h - the ABI's handle types and helpers, shared by the .cu files
// that implement include/qpe_gb300.h.
#ifndef QPE_ABI_INTERNAL_H_
#define QPE_ABI_INTERNAL_H_

#include <cuda_runtime.h>

#include <string>
#include <vector>

#include "../../include/qpe_gb300.h"
#include "kernels.h"
#include "program_build.h"
#include "qpe_common.h"

namespace qpe {

#define QPE_CK(expr)                                                                              \
  do {                                                                                            \
    cudaError_t e_ = (expr);                                                                      \
    if (e_ != cudaSuccess)                                                                        \
      throw ::qpe::Error(e_ == cudaErrorNoDevice || e_ == cudaErrorInsufficientDriver             \
                             ? QPE_ERR_NO_DEVICE                                                  \
                             : (e_ == cudaErrorMemoryAllocation ? QPE_ERR_NOMEM : QPE_ERR_CUDA),  \
                         std::string(#expr) + ": " + cudaGetErrorString(e_));                     \
  } while (0)

// Device buffer with RAII release.
struct DevBuf {
  void* p = nullptr;
  size_t bytes = 0;
  DevBuf() = default;
  DevBuf(const DevBuf&) = delete;
  DevBuf& operator=(const DevBuf&) = delete;
  ~DevBuf() { release(); }
  void release() {
    if (p) cudaFree(p);
    p = nullptr;
    bytes = 0;
  }
  void alloc(size_t n) {
    release();
    if (n == 0) n = 16;
    QPE_CK(cudaMalloc(&p, n));
    bytes = n;
  }
  template <class T>
  T* as() const {
    return reinterpret_cast<T*>(p);
  }
};

const std::string& last_error_message();

}  // namespace qpe

struct qpe_context {
  int device = 0;
  int num_sms = 0;
  size_t smem_optin = 0;
  cudaStream_t stream = nullptr;
  qpe::DevBuf binom;
  qpe::DevBuf flush;
  qpe::DevBuf err;  // device error word of the context's kernels (bounded waits)
  cudaEvent_t events[16] = {};
};

struct qpe_program {
  qpe_context* ctx = nullptr;
  uint64_t id = 0;  // unique per process, keys the cached evolution graphs
  qpe::HostProgram hp;
  qpe::DevBuf pool, ops, coef, strA, strB, tabs, start, passes;
  // MIX pass images (PassLaunch::img): all images back to back, and per pass
  // its first word and its length in words (0: no image).
  qpe::DevBuf images;
  std::vector<uint32_t> img_off, img_words;
  // Update-unit schedule of the column-pair passes (mix_units.h) for the lean
  // resident kernel, built on first use for one geometry (cluster, warps per
  // CTA, stage) and kept: mix_slot per pass, mix_words the warp programs.
  mutable qpe::DevBuf mix_words, mix_slot;
  mutable uint32_t mix_K = 0, mix_wpc = 0, mix_stage = 0, mix_wp_words = 0, mix_scheduled = 0;
  // Per-line programs of the row and column passes (mix_units.h) for one
  // geometry (cluster, warps per CTA, stage, rows per CTA, replicas).
  mutable qpe::DevBuf line_words, line_offs, line_slot;
  mutable uint32_t line_key[5] = {0, 0, 0, 0, 0}, line_passes = 0;
};

namespace qpe {
// Launch geometry of one pass of `pr` for elements of esz bytes.
PassLaunch plan_pass_geometry(const qpe_program* pr, size_t esz, size_t smem_optin, const Pass& pass);
std::vector<double> twiddle_table(uint32_t P);
void state_twiddles(uint32_t P, int dtype, DevBuf& tw);
void qift_geometry(uint32_t P, uint64_t ld, int dtype, int num_sms, size_t smem_optin, uint32_t& T, uint32_t& grid);
// Reads and clears the context's device error word (after the stream is
// synchronised); throws QPE_ERR_TIMEOUT if a kernel's bounded wait ran out.
void check_device_error(qpe_context* ctx);
}  // namespace qpe

#endif  // QPE_ABI_INTERNAL_H_
