// kernels.h - launch wrappers of the device kernels (kernels.cu, evolve.cu, qift.cu).
#ifndef QPE_KERNELS_H_
#define QPE_KERNELS_H_

#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/qpe_gb300.h"
#include "program.h"

namespace qpe {

// Binomial table with the reference nChoosek's values (cpp/util.hpp:49-60):
// BINOM_K columns per row, rows n = 0..63.
constexpr int BINOM_K = 65;
void host_ref_binom_table(uint64_t* out /* 64 * BINOM_K */);

cudaError_t launch_rank(const uint64_t* d_binom, const uint64_t* bvs, int64_t* ranks, size_t n, cudaStream_t s);
cudaError_t launch_unrank(const uint64_t* d_binom, uint32_t nbits, uint32_t weight, const int64_t* ranks,
                          uint64_t* bvs, size_t n, cudaStream_t s);
cudaError_t launch_rank_with_swaps(const uint64_t* d_binom, uint32_t nbits, uint64_t bv, const uint32_t* swaps,
                                   int64_t* out, size_t nq, cudaStream_t s);
// Strings of rank 0..count-1 (weight `weight` over `nbits` bits).
cudaError_t launch_line_strings(const uint64_t* d_binom, uint32_t nbits, uint32_t weight, uint32_t* out,
                                uint32_t count, cudaStream_t s);
cudaError_t launch_build_tables(const uint64_t* d_binom, const AxisTable* d_tabs, const uint32_t* d_entry_start,
                                uint32_t ntabs, uint64_t total_entries, uint32_t* d_pool, cudaStream_t s);

// FP64 FMA throughput probe (qpe_measure_fp64_peak): ctas x threads threads,
// kFp64ProbeChains independent FMA chains of `iters` steps each.
constexpr int kFp64ProbeChains = 8;
cudaError_t launch_fp64_fma_probe(double* out, uint32_t ctas, uint32_t threads, uint32_t iters, cudaStream_t s);

// ---- evolution (evolve.cu) ----
struct PassLaunch {
  void* work;                 // working block (Ca x Cb complex)
  const uint32_t* pool;
  const DevOp* ops;
  const double* coef;
  const uint32_t* strA;       // alpha strings by rank
  const uint32_t* strB;       // beta strings by rank
  uint32_t Ca, Cb;
  Pass pass;
  uint32_t W;                 // COL pass: lines per tile (power of two)
  uint32_t warps_per_cta;
  uint32_t grid;
  uint32_t exact;             // complex128: reference rounding (no contraction)
  uint32_t rev;               // run the pass's terms in reverse order
  // Batches: nmem instances sharing this program's structure. works[m] is member
  // m's working block (pl.work unused), icoef + m * nops its coefficients.
  void* const* works;
  const double2* icoef;
  uint32_t nmem, nops;
  // > 0: one tile per CTA of this many threads (a multiple of 32), which split
  // every term's entries (long tables); 0: one tile per warp.
  uint32_t cta_tile;
  // 1: column and column-pair tiles move between the working block and shared
  // memory as whole columns by bulk copies (cp.async.bulk, completing on an
  // mbarrier); needs every column to start on a 16-byte boundary (Ca * element
  // size a multiple of 16, working blocks 16-byte aligned).
  uint32_t bulk;
  // Device error word: a bounded wait that runs out ORs in kPassErrWait.
  int* err;
  // A MIX pass's image (with bulk): its term descriptors followed by the tables
  // they use, the descriptors' table offsets relative to the image, img_words
  // 32-bit words (a multiple of 4); each CTA brings it into shared memory with
  // one bulk copy, so the term setup reads at shared-memory latency. nullptr:
  // descriptors and tables are read from the program in global memory.
  const uint32_t* img;
  uint32_t img_words;
};
constexpr int kPassErrWait = 2;
// Largest pass image (bytes) a pass launch stages in shared memory.
constexpr uint32_t kPassImageMaxBytes = 48 * 1024;
// Dynamic shared memory of a pass launch: its tile stages and its image.
size_t pass_smem_bytes(const PassLaunch& pl, size_t esz);
// One run of words copied from the program's index pool into a pass image.
struct PassImageSeg {
  uint32_t src, dst, words;
};
cudaError_t launch_copy_segments(const uint32_t* src, uint32_t* dst, const PassImageSeg* segs, uint32_t n,
                                 cudaStream_t s);
constexpr uint32_t kCtaTileThreads = 128;
size_t pass_stage_elems(const Pass& pass, uint32_t Ca, uint32_t Cb, uint32_t W);
cudaError_t launch_pass(const PassLaunch& pl, int dtype, cudaStream_t s);
// The tile passes' working block is stored by columns (element (a, b) at
// b * Ca + a); the register keeps row-major blocks. Snapshot: working block ->
// block *d_k of the register; load: block `block` -> working block.
cudaError_t launch_snapshot(const void* work, void* state, uint32_t Ca, uint32_t Cb, const int* d_k, int dtype,
                            cudaStream_t s);
cudaError_t launch_load(void* work, const void* state, uint32_t Ca, uint32_t Cb, uint32_t block, int dtype,
                        cudaStream_t s);
cudaError_t launch_advance(int* d_k, cudaStream_t s);
// Batches: the same for every member of a class.
cudaError_t launch_snapshot_batch(void* const* works, void* const* states, uint32_t Ca, uint32_t Cb, const int* d_k,
                                  uint32_t nmem, int dtype, cudaStream_t s);
cudaError_t launch_load_batch(void* const* works, void* const* states, uint32_t Ca, uint32_t Cb, uint32_t block,
                              uint32_t nmem, int dtype, cudaStream_t s);
// Sets the graph's while-loop condition to (*d_k + 1 < last).
cudaError_t launch_continue_while(const int* d_k, int last, cudaGraphConditionalHandle h, cudaStream_t s);
cudaError_t configure_pass_kernels(int dtype, size_t smem_bytes);

// ---- resident evolution (resident.cu) ----
// One instance of the resident kernel: its register in global memory and its
// compiled program. Lines per tile Wc / Wr / Wm are powers of two dividing 32.
struct ResidentInstance {
  void* state;
  const uint32_t* pool;
  const DevOp* ops;
  const double* coef;
  const Pass* passes;
  const uint32_t* strA;
  const uint32_t* strB;
  uint32_t Ca, Cb, npasses;
  uint32_t first, last;     // powers evolved: blocks first .. last - 1
  uint32_t rows_per_cta;    // rows owned by each CTA of the cluster
  uint32_t Wc, Wr, Wm;
  uint32_t steps, order;    // Trotter steps per power; 2 = forward + backward sweep
  uint32_t nops, pool_words;  // sizes of the term descriptors and the index pool
  uint32_t in_place;        // 1: block `first` is loaded, evolved last - first times
                            //    and written back to itself (iterative QPE)
  // Column-pair passes as update units (mix_units.h; k_resident_lean only): the
  // warp programs, per pass its block of them or kMixNoSchedule, and the words
  // of one program. mix_words == nullptr: every column-pair pass by tiles.
  const uint32_t* mix_words;
  const uint32_t* mix_slot;
  uint32_t mix_wp_words;
  // Replicas (k_resident_lean, cluster > 1): `replicas` clusters each hold the
  // whole block. Row and column passes are split between them (rows, columns by
  // index modulo replicas) and every cluster takes the others' results through
  // xbuf (two blocks, by exchange parity); xflag holds one exchange count per
  // (replica, CTA), zero at launch. Column-pair passes run on every replica.
  // replicas <= 1: one cluster. A wait for another replica that runs out ORs
  // kResidentErrExchange into *err and the CTA stops waiting.
  uint32_t replicas;
  void* xbuf;
  uint32_t* xflag;
  int* err;
  // Row and column passes as per-line programs (mix_units.h, k_resident_lean
  // with a cluster > 1): per pass its block of program offsets or
  // kMixNoSchedule, the offsets ([block][replica][cta][warp]) and the programs.
  // line_slot == nullptr: every row and column pass by the line runner.
  const uint32_t* line_slot;
  const uint32_t* line_offs;
  const uint32_t* line_words;
};
constexpr int kResidentErrExchange = 4;
struct ResidentLaunch {
  const ResidentInstance* insts;  // device array, ninst entries
  uint32_t ninst;
  uint32_t cluster;               // CTAs per instance (1 = one CTA)
  uint32_t warps_per_cta;
  uint32_t stage_elems;           // per-warp stage (cluster > 1)
  uint32_t group;                 // 1: four-warp tile groups with quad-split updates
                                  //    (k_resident_group); stage_elems is then per group
                                  // 2: column-pair passes by four-warp groups (whose
                                  //    stage is their four warps' stages), row and
                                  //    column passes by single warps (k_resident)
                                  // 3: every tile by a three-warp group (k_resident_lean);
                                  //    stage_elems is per group
  uint32_t meta_smem;             // 1: term descriptors, index pool, passes and line
                                  //    strings are staged in every CTA's shared memory
  uint32_t replicas;              // clusters per instance (k_resident_lean; 0 or 1: one),
                                  // launched cooperatively when more than one
  size_t smem_bytes;
};
// Upper bound of the resident kernels' static shared memory (a scratch element
// per four-warp group).
constexpr size_t kResidentStaticSmem = 256;
// Bytes of shared memory the staged program metadata takes (ResidentLaunch::meta_smem).
size_t resident_meta_bytes(uint32_t nops, uint32_t pool_words, uint32_t npasses, uint32_t Ca, uint32_t Cb);
cudaError_t launch_resident(const ResidentLaunch& rl, int dtype, int exact, cudaStream_t s);
// Shared-memory carveout (percent of the maximum) the resident kernel asks for.
cudaError_t set_resident_carveout(int dtype, int exact, int percent);

// ---- QIFT and reductions (qift.cu) ----
cudaError_t launch_qift(void* state, uint64_t ld, uint32_t P, const void* twiddles, double norm, double* partial,
                        uint32_t grid, uint32_t cols_per_cta, int dtype, cudaStream_t s);
size_t qift_smem_bytes(uint32_t P, uint32_t cols_per_cta, int dtype);
cudaError_t configure_qift_kernels(int dtype, size_t smem_bytes);
cudaError_t launch_reduce_partials(const double* partial, uint32_t nparts, uint32_t N, double* out, cudaStream_t s);
cudaError_t launch_block_sums(const void* state, uint64_t ld, uint32_t N, double* out, int dtype, cudaStream_t s);

}  // namespace qpe

#endif  // QPE_KERNELS_H_
