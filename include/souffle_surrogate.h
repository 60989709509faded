/*
 * Learned far-field surrogate for the inter-subunit interaction: a small MLP trained and run with
 * BF16 tensor-core (tcgen05) kernels.  None of these entry points has a counterpart in the
 * reference, which has no learned part; they extend the force path of souffle_gpu.h.
 *
 * Network: n_in -> width -> width -> width -> n_out, SiLU after each hidden layer, BF16 weights
 * and activations, FP32 accumulation, FP32 master weights updated by Adam.  Loss: mean squared
 * error over the n_out outputs.
 *
 * Device-pointer arguments (suffix _dev) are row-major FP32 arrays in the handle's device memory;
 * calls run on the handle's stream and return once their results are ready.
 */
#ifndef SOUFFLE_SURROGATE_H
#define SOUFFLE_SURROGATE_H

#include <stdint.h>

#include "souffle_gpu.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct souffle_mlp souffle_mlp;

/* n_in a multiple of 8 up to 256, n_out at most 256, width 256 (the hidden layers are one 256-wide tensor-core tile),
 * max_batch rows per call (rounded up to 128 internally).  Weights are initialised from seed
 * (uniform, +-sqrt(3 / fan_in)), biases zero. */
souffle_status souffle_mlp_create(int32_t n_in, int32_t width, int32_t n_out, int32_t max_batch, uint64_t seed,
                                  int32_t device, souffle_mlp** out);
souffle_status souffle_mlp_destroy(souffle_mlp* h);

/* Number of FP32 parameters, flat layout W1 [width][n_in], b1 [width], W2, b2, W3, b3,
 * W4 [n_out][width], b4 [n_out]. */
int64_t souffle_mlp_param_count(const souffle_mlp* h);
souffle_status souffle_mlp_get_params(souffle_mlp* h, float* host_out, int64_t n);
souffle_status souffle_mlp_set_params(souffle_mlp* h, const float* host_in, int64_t n);

/* y_dev [m][n_out] = network(x_dev [m][n_in]); 1 <= m <= max_batch. */
souffle_status souffle_mlp_forward(souffle_mlp* h, const float* x_dev, int32_t m, float* y_dev);

/* Loss and gradient of the loss with respect to every parameter (flat layout above, host array
 * of souffle_mlp_param_count floats) for one batch; parameters unchanged. */
souffle_status souffle_mlp_gradients(souffle_mlp* h, const float* x_dev, const float* t_dev, int32_t m,
                                     float* loss, float* grad_host);

/* One Adam step (beta1 0.9, beta2 0.999, eps 1e-8) on one batch; *loss is the batch loss before
 * the step. */
souffle_status souffle_mlp_train_step(souffle_mlp* h, const float* x_dev, const float* t_dev, int32_t m, float lr,
                                      float* loss);

/* Utility: C [m][n] FP32 = A [m][k] * B [n][k]^T with A, B given as FP32 device arrays, rounded to
 * BF16 and multiplied on the tensor cores (FP32 accumulation).  For tests of the GEMM itself. */
souffle_status souffle_gemm_bf16(const float* a_dev, const float* b_dev, int32_t m, int32_t n, int32_t k,
                                 float* c_dev, int32_t device);

#ifdef __cplusplus
}
#endif

#endif
