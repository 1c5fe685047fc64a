/*
 * qpe_gb300_mlp.h - C ABI of the learned initial-state model.
 *
 * An MLP over occupation bit strings proposes the amplitudes of the QPE initial
 * state in place of Hartree-Fock: n_bits inputs (bit j of the string as 0 / 1),
 * optionally followed by n_feat real features of the string (qpe_mlp_create2),
 * three hidden layers of 256 with GELU, outputs (log|a|, phase). BF16 weights and
 * activations with FP32 accumulation on the tensor cores (tcgen05 MMA, TMA
 * operand loads); FP32 master weights, Adam moments and loss.
 *
 * The reference has no counterpart: this is an extension beside the hot path. The
 * state it proposes enters the evolution through qpe_state_upload as block 0.
 */
#ifndef QPE_GB300_MLP_H_
#define QPE_GB300_MLP_H_

#include <stddef.h>
#include <stdint.h>

#include "qpe_gb300.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct qpe_mlp qpe_mlp;

/* A model with seeded initial weights; `batch` (a multiple of 128) is the number
 * of samples per training step and per forward chunk. */
int qpe_mlp_create(qpe_context* ctx, uint32_t n_bits, uint32_t batch, uint64_t seed, qpe_mlp** out);
/* The same with n_feat extra real input features per sample after the n_bits
 * occupations (n_bits + n_feat <= 64), e.g. quantities of the Hamiltonian the
 * string belongs to; the *2 calls below then take them, n_feat floats per sample. */
int qpe_mlp_create2(qpe_context* ctx, uint32_t n_bits, uint32_t n_feat, uint32_t batch, uint64_t seed,
                    qpe_mlp** out);
int qpe_mlp_destroy(qpe_mlp* m);

/* Parameters as one FP32 array, in this order: W1 [256 x 64] (input columns past
 * n_bits are zero), b1 [256], W2 [256 x 256], b2 [256], W3 [256 x 256], b3 [256],
 * W4 [16 x 256] (rows past 1 are zero), b4 [16] (entries past 1 are zero). */
int qpe_mlp_num_params(const qpe_mlp* m, uint64_t* n);
int qpe_mlp_get_params(qpe_mlp* m, float* host);
int qpe_mlp_set_params(qpe_mlp* m, const float* host);

/* Training set, copied to the device: per sample the occupation string, the
 * target log|a|, phase, and the loss weight. */
int qpe_mlp_set_data(qpe_mlp* m, const uint64_t* bits, const float* log_abs, const float* phase,
                     const float* weight, uint64_t count);
int qpe_mlp_set_data2(qpe_mlp* m, const uint64_t* bits, const float* feats, const float* log_abs, const float* phase,
                      const float* weight, uint64_t count);

/* `steps` Adam steps (learning rate lr) on batches drawn from the training set
 * with a seeded hash; losses (may be NULL) receives each step's loss:
 * (1 / batch) sum_b w_b [(log|a|_b - t_b)^2 + (1 - cos(phase_b - p_b))]. */
int qpe_mlp_train(qpe_mlp* m, uint32_t steps, float lr, uint64_t seed, float* losses);

/* Model outputs for `count` strings: out[2 i] = log|a|, out[2 i + 1] = phase. */
int qpe_mlp_forward(qpe_mlp* m, const uint64_t* bits, uint64_t count, float* out);
int qpe_mlp_forward2(qpe_mlp* m, const uint64_t* bits, const float* feats, uint64_t count, float* out);

/* Loss and gradient of every parameter (the qpe_mlp_get_params layout) on one
 * batch of `count` <= batch samples, without an update. */
int qpe_mlp_gradients(qpe_mlp* m, const uint64_t* bits, const float* log_abs, const float* phase,
                      const float* weight, uint32_t count, float* grads, float* loss);
int qpe_mlp_gradients2(qpe_mlp* m, const uint64_t* bits, const float* feats, const float* log_abs,
                       const float* phase, const float* weight, uint32_t count, float* grads, float* loss);

/* Tensor-core FLOPs of one training step (the 11 GEMMs). */
int qpe_mlp_tensor_flops_per_step(const qpe_mlp* m, double* flops);

/* The tensor-core GEMM alone: D[M, N] (FP32) = A[M, K] . B[N, K]^T with A, B
 * row-major BF16 (as uint16 bit patterns); M % 128 == 0, K % 64 == 0,
 * N % tile_n == 0, tile_n in {16, 64, 256}. */
int qpe_gemm_bf16(qpe_context* ctx, uint32_t M, uint32_t N, uint32_t K, const uint16_t* A, const uint16_t* B,
                  float* D, uint32_t tile_n);

#ifdef __cplusplus
}
#endif
#endif /* QPE_GB300_MLP_H_ */
