/*
 * qpe_gb300.h - C ABI of the GB300 (sm_103a) implementation of qpe-sim's hot path:
 * the controlled, Trotterized time evolution of a fixed-electron-count state vector
 * followed by the batched inverse QFT over the ancilla axis.
 *
 * Every entry point returns an int status (QPE_OK == 0). No C++ exception crosses
 * this boundary; qpe_last_error() returns a thread-local message for the last
 * failing call on the calling thread.
 *
 * State layout (identical to the reference StateVector, cpp/state_vector.hpp:20-42):
 *   amplitude(k, a, b) at index k * Ca * Cb + a * Cb + b,
 *   k in [0, 2^P) the ancilla value, a = OffsetComputer::rank of the alpha string,
 *   b = rank of the beta string, Ca = C(M, Na), Cb = C(M, Nb).
 *   Host buffers are interleaved (re, im) doubles (std::complex<double>) or floats.
 * Spin-orbital indices follow SpinIndex::HalfUp (cpp/types.hpp:50-55):
 *   alpha orbital o -> o, beta orbital o -> M + o (0-based).
 */
#ifndef QPE_GB300_H_
#define QPE_GB300_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------ */
#define QPE_OK 0
#define QPE_ERR_INVALID 1     /* bad shape, index or argument */
#define QPE_ERR_UNSUPPORTED 2 /* shape outside what the library handles */
#define QPE_ERR_NOMEM 3       /* device or host allocation failed */
#define QPE_ERR_CUDA 4        /* a CUDA runtime call failed */
#define QPE_ERR_TIMEOUT 5     /* a bounded device-side wait gave up */
#define QPE_ERR_NO_DEVICE 6   /* no usable CUDA device */

/* ---- state element types ------------------------------------------------ */
#define QPE_C128 0 /* complex double: the reference's std::complex<double> */
#define QPE_C64 1  /* complex float state, FP64 coefficients and reductions */

/* ---- term kinds (the five segments of
 *      Hamiltonian::PrintIndexedSegmentedHamiltonianTerms, cpp/hamiltonian.cc:253-299) */
#define QPE_TERM_PP 0
#define QPE_TERM_PQ 1
#define QPE_TERM_PQQP 2
#define QPE_TERM_PQQR 3
#define QPE_TERM_PQRS 4

/*
 * One indexed Hamiltonian term with its host-computed exponentiated coefficients.
 *   pp   : key (p, p)        coefficient Hamiltonian::pp_term(p)        -> even[0..1]
 *   pq   : key (p, q), p > q  pq_term(p, q, parity)                       -> even / odd
 *   pqqp : key (p, q, q, p)   pqqp_term(p, q)                             -> even[0..1]
 *   pqqr : key (p, q, q, r)   pqqr_term(p, q, r, parity)                  -> even / odd
 *   pqrs : key (p, q, r, s)   pqrs_term(p, q, r, s, parity)               -> even / odd
 * even/odd hold {m00.re, m00.im, m01.re, m01.im} of the symmetric 2x2 matrix
 * [[m00, m01], [m01, m00]] for JW parity 0 / 1 (cpp/hamiltonian.cc:674-783).
 * Diagonal terms use even[0], even[1] only. Unused indices are ignored.
 */
typedef struct qpe_term {
  uint32_t p, q, r, s;
  double even[4];
  double odd[4];
} qpe_term;

/* ---- context -------------------------------------------------------------- */
typedef struct qpe_context qpe_context;

int qpe_version(void);
const char* qpe_last_error(void);
int qpe_device_count(int* count);
int qpe_context_create(int device, qpe_context** out);
int qpe_context_destroy(qpe_context* ctx);
int qpe_synchronize(qpe_context* ctx);

/* CUDA events on the context's stream (slots 0..15), for timing the library's
 * own work on the stream it launches on. */
int qpe_timer_record(qpe_context* ctx, uint32_t slot);
int qpe_timer_elapsed_ms(qpe_context* ctx, uint32_t start_slot, uint32_t end_slot, float* ms);

/* Measures the device's FP64 FMA throughput (TFLOP/s, an FMA counting 2): a
 * kernel of 8 independent FMA chains per thread on 4 x 256-thread CTAs per SM,
 * timed with CUDA events of its own on the context's stream. A
 * measurement helper for reporting FP64 roofline fractions; no counterpart in
 * the reference. */
int qpe_measure_fp64_peak(qpe_context* ctx, double* tflops);

/* Page-locked host memory (cudaMallocHost), for host buffers the copies of
 * the one-shot and resident APIs read and write at full speed. */
int qpe_host_alloc(size_t bytes, void** out);
int qpe_host_free(void* p);

/* Writes a 256 MiB device buffer (allocated on first use) so that the next
 * timed region starts with nothing of the state in L2. */
int qpe_flush_l2(qpe_context* ctx);

/* Self-test of the bounded device waits (no counterpart in the reference, which
 * only asserts: cpp/offset_computer.hpp:39,47). Every wait of the library's
 * tcgen05 / TMA kernels polls an mbarrier a bounded number of times, and a wait
 * that runs out makes the kernel record an error and return, so the call reports
 * QPE_ERR_TIMEOUT and the context stays usable. This runs that wait alone on one
 * mbarrier with nothing else in flight: with arrive = 0 nobody completes it, the
 * wait gives up after max_tries polls and the call returns QPE_ERR_TIMEOUT; with
 * arrive = 1 a thread completes it first and the call returns QPE_OK. */
int qpe_selftest_bounded_wait(qpe_context* ctx, uint32_t max_tries, int arrive);

/* ---- combinatorial primitives (device kernels) ------------------------------ */

/* Replaces OffsetComputer::rank (cpp/offset_computer.hpp:16-27): colex rank
 * sum_i C(pos_i, i + 1) over the set bits of each bit vector. Host arrays. */
int qpe_rank(qpe_context* ctx, const uint64_t* bvs, int64_t* ranks, size_t n);

/* Inverse of qpe_rank over the weight-`weight` strings of `nbits` bits (the
 * enumeration order of next_comb, cpp/util.hpp:62-70). Host arrays. */
int qpe_unrank(qpe_context* ctx, uint32_t nbits, uint32_t weight, const int64_t* ranks,
               uint64_t* bvs, size_t n);

/* Replaces OffsetComputer(n, bv, rank).rank_with_swap(i, j) and
 * .rank_with_double_swap(i, j, k, l) (cpp/offset_computer.hpp:128-192) for a
 * batch of queries against one bit vector; computed on the device from prefix
 * tables. `swaps` holds n_queries rows of 4 positions; for a single swap set
 * the last two to 0xFFFFFFFF. */
int qpe_rank_with_swaps(qpe_context* ctx, uint32_t nbits, uint64_t bv, const uint32_t* swaps,
                        int64_t* ranks, size_t n_queries);

/* Replaces the discover*_BVs routines (cpp/time_evolution_over_terms.hpp:1160-1411)
 * for one term on one spin: builds the index table on the device and returns it
 * with the runs expanded, entry j being the j-th string of the reference's run
 * order. kind: 0 N(q), 1 NN(p, r), 2 CA(p, r), 3 CNA(p, q, r), 4 CCAA(p, q, r, s);
 * orbitals holds those orbitals in that order (0-based within the spin). For the
 * list kinds (N, NN) i10 is left untouched and parity is 0. *count receives the
 * number of entries; cap bounds the output arrays. */
int qpe_axis_table(qpe_context* ctx, int kind, uint32_t nbits, uint32_t weight, const uint32_t* orbitals,
                   uint32_t* i01, uint32_t* i10, uint8_t* parity, size_t cap, size_t* count);

/* ---- one-shot calls shaped like the reference's (host buffers) -------------- */

/* Replaces time_evolve_over_terms(StateVector&, Hamiltonian&, unsigned precision)
 * (cpp/time_evolution_over_terms.hpp:92-139). The five arrays are the segmented
 * indexed terms in map order with their coefficients; the library applies them in
 * the order of applyUnitary_reordered (:374-562), including the nesting of pqqr
 * terms under their pq term and the skipping rule of :465. `state` holds
 * 2^precision * C(M, num_occupied)^2 interleaved complex doubles with block 0
 * filled; on return every block k holds U^k * block 0. */
int qpe_time_evolve_over_terms(qpe_context* ctx, uint32_t num_orbitals, uint32_t num_occupied,
                               uint32_t precision, const qpe_term* pp, size_t n_pp,
                               const qpe_term* pq, size_t n_pq, const qpe_term* pqqp,
                               size_t n_pqqp, const qpe_term* pqqr, size_t n_pqqr,
                               const qpe_term* pqrs, size_t n_pqrs, double* state);

/* Replaces time_evolve_iqpe(StateVector&, Hamiltonian&, unsigned num_of_applications)
 * (cpp/time_evolution_over_terms.hpp:141-155): block 1 of `state` (2^precision
 * blocks, precision >= 1) receives num_of_applications sweeps of applyUnitary
 * (:174-372) in place; the other blocks are left as they are. */
int qpe_time_evolve_iqpe(qpe_context* ctx, uint32_t num_orbitals, uint32_t num_occupied, uint32_t precision,
                         const qpe_term* pp, size_t n_pp, const qpe_term* pq, size_t n_pq,
                         const qpe_term* pqqp, size_t n_pqqp, const qpe_term* pqqr, size_t n_pqqr,
                         const qpe_term* pqrs, size_t n_pqrs, uint32_t num_of_applications,
                         double* state);

/* Replaces StateVector::qift() (cpp/state_vector.hpp:115-179): in-place forward
 * DFT (sign -1) of length 2^precision along the ancilla axis (stride ld, ld
 * transforms), then division by sqrt(2^precision). */
int qpe_qift(qpe_context* ctx, uint32_t precision, uint64_t ld, double* state);

/* Replaces StateVector::IdentifyPhaseAmplitudes() (cpp/state_vector.hpp:341-372):
 * probs[k] = sum over the block of |amplitude(k, .)|^2. */
int qpe_identify_phase_amplitudes(qpe_context* ctx, uint32_t precision, uint64_t ld,
                                  const double* state, double* probs);

/* ---- device-resident API --------------------------------------------------- */

typedef struct qpe_program qpe_program; /* compiled term program of one Hamiltonian */
typedef struct qpe_state qpe_state;     /* device-resident 2^P x Ca x Cb state */

typedef struct qpe_program_info {
  uint32_t num_orbitals, n_alpha, n_beta;
  uint32_t c_alpha, c_beta;
  uint32_t num_ops;          /* term applications in one Trotter sweep */
  uint32_t num_ops_per_power;
  uint64_t touches_per_sweep; /* amplitude-term updates in one sweep (pair = 2, diagonal = 1) */
  uint64_t touches_per_power;
  uint64_t table_entries;     /* device index-table entries */
  uint32_t num_passes_per_power; /* tile passes (kernel launches) per controlled power */
  uint32_t reserved;
} qpe_program_info;

/* Term order, or-ed into trotter_order of qpe_program_create / qpe_program_plan:
 * the order of applyUnitary (cpp/time_evolution_over_terms.hpp:174-372), used by
 * time_evolve_iqpe: every pp, then every pq, pqqp, pqqr (none skipped) and pqrs
 * term, instead of applyUnitary_reordered's pq-with-nested-pqqr order. */
#define QPE_PROGRAM_APPLY_UNITARY_ORDER 0x100u

/* Builds the application order and the device pair tables for one Hamiltonian.
 * n_alpha == n_beta reproduces the reference; n_alpha != n_beta is an extension
 * (odd electron counts) the reference cannot represent.
 * trotter_order 1 = the reference's first-order sweep; 2 = symmetric (Strang)
 * product of a forward and a reversed sweep, each with the coefficients given
 * (compute them at half the step). steps_per_power repeats the step.
 * A program keeps the schedules QPE_STRATEGY_LEAN_UNITS builds on first use
 * (for one cluster, replica count and geometry at a time): evolve with one
 * program from one host thread at a time. */
int qpe_program_create(qpe_context* ctx, uint32_t num_orbitals, uint32_t n_alpha,
                       uint32_t n_beta, const qpe_term* pp, size_t n_pp, const qpe_term* pq,
                       size_t n_pq, const qpe_term* pqqp, size_t n_pqqp, const qpe_term* pqqr,
                       size_t n_pqqr, const qpe_term* pqrs, size_t n_pqrs, uint32_t trotter_order,
                       uint32_t steps_per_power, qpe_program** out);
int qpe_program_destroy(qpe_program* prog);
/* Host-only planning of the same program (no device work): fills *info. */
int qpe_program_plan(uint32_t num_orbitals, uint32_t n_alpha, uint32_t n_beta, const qpe_term* pp, size_t n_pp,
                     const qpe_term* pq, size_t n_pq, const qpe_term* pqqp, size_t n_pqqp, const qpe_term* pqqr,
                     size_t n_pqqr, const qpe_term* pqrs, size_t n_pqrs, uint32_t trotter_order,
                     uint32_t steps_per_power, qpe_program_info* info);
int qpe_program_get_info(const qpe_program* prog, qpe_program_info* info);
/* The column-pair update-unit schedule (QPE_STRATEGY_LEAN_UNITS) the program last
 * built: its cluster size and how many column-pair passes it schedules (the rest
 * run as tiles); 0, 0 before any evolution with that strategy. */
int qpe_program_unit_schedule(const qpe_program* prog, uint32_t* cluster_size, uint32_t* scheduled_passes);

int qpe_state_create(qpe_context* ctx, uint32_t num_orbitals, uint32_t n_alpha, uint32_t n_beta,
                     uint32_t precision, int dtype, qpe_state** out);
int qpe_state_destroy(qpe_state* st);
/* Host <-> device copies of elements [first, first + count) of the state, in the
 * state's element type (interleaved doubles for QPE_C128, floats for QPE_C64). */
int qpe_state_upload(qpe_state* st, const void* host, uint64_t first, uint64_t count);
int qpe_state_download(qpe_state* st, void* host, uint64_t first, uint64_t count);
int qpe_state_zero(qpe_state* st);

#define QPE_STRATEGY_AUTO 0
#define QPE_STRATEGY_RESIDENT 1 /* whole block in one CTA's shared memory */
#define QPE_STRATEGY_CLUSTER 2  /* block spread over a thread-block cluster */
#define QPE_STRATEGY_TILED 3    /* L2-resident block, shared-memory tile passes */
#define QPE_STRATEGY_GROUP 4    /* as CLUSTER (cluster_size 1..16), tiles processed by four-warp
                                   groups with every update split over four lanes */
#define QPE_STRATEGY_HYBRID 5   /* as CLUSTER (cluster_size 1..16): column-pair passes as GROUP,
                                   row and column passes as CLUSTER */
#define QPE_STRATEGY_LEAN 6     /* as CLUSTER (cluster_size 1..16): every row, column or column
                                   pair processed by a three-warp group, pair updates split over
                                   four lanes and diagonal updates over two */
#define QPE_STRATEGY_LEAN_UNITS 7 /* as LEAN (cluster_size 2..16), with runs of column-pair passes
                                     split into the connected components of their pairings
                                     (update units) packed into warps by a host schedule, and the
                                     row and column passes run as per-line programs whose term
                                     conditions the host evaluated: no CTA runs two column pairs
                                     while others idle, one gather, scatter and cluster barrier per
                                     window of up to 8 passes, no per-term decisions on the device */

/* complex128 only: allow fused multiply-adds. Results then differ from the
 * reference's rounding by a few ulps per update (within 1e-12 of it) instead of
 * being bit-identical, for about a third fewer FP64 instructions. */
#define QPE_EVOLVE_FP64_CONTRACT 1u
/* time_evolve_iqpe (cpp/time_evolution_over_terms.hpp:141-155): block first_power is
 * evolved in place, `repeats` times (0 = once), with no copy from the block before
 * it; last_power is ignored. With a program built in the applyUnitary term order
 * (QPE_PROGRAM_APPLY_UNITARY_ORDER) and first_power = 1 this is the reference's
 * iterative-QPE evolution. */
#define QPE_EVOLVE_IN_PLACE 2u

typedef struct qpe_evolve_opts {
  uint32_t strategy;     /* QPE_STRATEGY_* */
  uint32_t first_power;  /* evolve blocks first_power .. last_power - 1 (0, 0 = all) */
  uint32_t last_power;
  uint32_t cluster_size; /* QPE_STRATEGY_CLUSTER: CTAs per cluster (0 = auto) */
  uint32_t flags;        /* QPE_EVOLVE_* */
  uint32_t repeats;      /* QPE_EVOLVE_IN_PLACE: applications of the power (0 = 1) */
  uint32_t replicas;     /* QPE_STRATEGY_LEAN_UNITS: clusters that each hold the whole block
                            and split the row and column passes between them, exchanging
                            their results through global memory (0 or 1: one cluster; at
                            most 8; launched cooperatively). The autotuner tries 1 to 5. */
} qpe_evolve_opts;

/* block_k <- U * block_{k-1} for k = 1 .. 2^P - 1 on the device (opts may be NULL). */
int qpe_evolve(qpe_state* st, const qpe_program* prog, const qpe_evolve_opts* opts);
/* In-place QIFT of the device state; also records the phase histogram. */
int qpe_state_qift(qpe_state* st);
/* Phase histogram (2^P doubles) of the device state, computed in FP64. */
int qpe_state_phase_probs(qpe_state* st, double* probs);
/* Per-block squared norms (2^P doubles, FP64 accumulation). */
int qpe_state_block_norms(qpe_state* st, double* norms);
/* Strategy (QPE_STRATEGY_*) and cluster size the last qpe_evolve on this state ran. */
int qpe_state_last_strategy(const qpe_state* st, uint32_t* strategy, uint32_t* cluster_size);
/* Replica clusters (qpe_evolve_opts::replicas) the last qpe_evolve on this state ran. */
int qpe_state_last_replicas(const qpe_state* st, uint32_t* replicas);

/* ---- batching form ----------------------------------------------------------------
 * Many Hamiltonians (programs) evolved, transformed and read out by one launch of
 * one CUDA graph. Instances whose programs have the same structure share index
 * tables and term lists; each keeps its own coefficients and its own 2^P x Ca x Cb
 * register. No counterpart in the reference (which runs one Hamiltonian). */
typedef struct qpe_batch qpe_batch;
typedef struct qpe_batch_info {
  uint32_t instances, classes;
  uint64_t touches_per_run;  /* amplitude-term updates of one qpe_batch_run */
  uint64_t amplitudes;       /* register elements over all instances */
  uint32_t launches_per_run; /* kernel launches one run makes inside its graph */
  uint32_t reserved;
} qpe_batch_info;
int qpe_batch_create(qpe_context* ctx, uint32_t n, const qpe_program* const* programs, uint32_t precision,
                     int dtype, qpe_batch** out);
int qpe_batch_destroy(qpe_batch* b);
int qpe_batch_upload(qpe_batch* b, uint32_t instance, const void* host, uint64_t first, uint64_t count);
int qpe_batch_download(qpe_batch* b, uint32_t instance, void* host, uint64_t first, uint64_t count);
/* Times one power of every candidate tile shape per class and keeps the fastest. */
int qpe_batch_tune(qpe_batch* b);
/* One graph launch: every power of every instance, then every QIFT and histogram.
 * Blocks 1.. of each register are overwritten from its block 0. */
int qpe_batch_run(qpe_batch* b, int synchronize);
int qpe_batch_phase_probs(qpe_batch* b, uint32_t instance, double* probs);
int qpe_batch_get_info(const qpe_batch* b, qpe_batch_info* info);
/* One class of a batch: instances of one program structure (one (M, Na, Nb)
 * for the synthetic generator). ms_per_power is the tuned time of one power of
 * the whole class run alone (measured by qpe_batch_tune; 0 before it). */
typedef struct qpe_batch_class {
  uint32_t num_orbitals, n_alpha, n_beta, members;
  uint64_t touches_per_power;  /* summed over the class's members */
  float ms_per_power;
  uint32_t tile_lines, warps_per_cta;  /* the tuned tile shape (warps_per_cta 0: one tile per CTA) */
} qpe_batch_class;
int qpe_batch_class_info(const qpe_batch* b, uint32_t cls, qpe_batch_class* out);

/* ---- QIFT without any allocation ------------------------------------------------
 * No counterpart in the reference. For callers that cannot let a library allocate
 * device memory: a host application that hands out all device memory from its own
 * pool and forbids libraries from taking more, or a latency-bound loop that cannot
 * afford cudaMalloc / cudaFree (which may synchronise the device). Runs the QIFT of
 * qpe_state_qift in place on the caller's device register d_state (2^precision x
 * ld elements of dtype) on the caller's cudaStream_t `stream` and writes the phase
 * histogram (2^precision doubles) to the device buffer d_probs. It calls no
 * allocator: the kernel's scratch (histogram partial rows, about 2 MiB) and the
 * twiddle tables of every precision (24 KiB) are fixed arrays inside the library,
 * which every GPU that loads the library holds until the process exits; precision
 * above QPE_NOALLOC_MAX_PRECISION is rejected with QPE_ERR_UNSUPPORTED. The first
 * call on a device, with that device current, does the set-up: it looks up the
 * arrays' device addresses (cudaGetSymbolAddress), fills the twiddle tables with a
 * synchronous copy and sets the QIFT kernel's shared-memory limit; make that first
 * call before any stream capture. Later calls only launch kernels on `stream`.
 * All calls share the partial rows: calls that overlap on the GPU (other streams,
 * other host threads) race on them. */
#define QPE_NOALLOC_MAX_PRECISION 10
#define QPE_NOALLOC_MAX_CTAS 256
#define QPE_NOALLOC_SCRATCH_DOUBLES ((QPE_NOALLOC_MAX_CTAS << QPE_NOALLOC_MAX_PRECISION) + (1 << QPE_NOALLOC_MAX_PRECISION))
int qpe_qift_device_noalloc(void* stream, uint32_t precision, uint64_t ld, int dtype, void* d_state,
                            double* d_probs);

#ifdef __cplusplus
}
#endif
#endif /* QPE_GB300_H_ */
