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

/* n_in a multiple of 8 up to 256, n_out at most 256, width 128 or 256 (a hidden layer is one or two 128-wide
 * tensor-core tiles), max_batch rows per call (rounded up to 128 internally).  Weights are initialised from seed
 * (uniform, +-sqrt(3 / fan_in)), biases zero. */
souffle_status souffle_mlp_create(int32_t n_in, int32_t width, int32_t n_out, int32_t max_batch, uint64_t seed,
                                  int32_t device, souffle_mlp** out);
souffle_status souffle_mlp_destroy(souffle_mlp* h);
/* The network's CUDA stream (cudaStream_t), on which its calls run, for callers that order or
 * time their own work against it. */
void* souffle_mlp_stream(const souffle_mlp* h);

/* Number of FP32 parameters, flat layout W1 [width][n_in], b1 [width], W2, b2, W3, b3,
 * W4 [n_out][width], b4 [n_out]. */
int64_t souffle_mlp_param_count(const souffle_mlp* h);
souffle_status souffle_mlp_get_params(souffle_mlp* h, float* host_out, int64_t n);
souffle_status souffle_mlp_set_params(souffle_mlp* h, const float* host_in, int64_t n);

/* y_dev [m][n_out] = network(x_dev [m][n_in]); 1 <= m <= max_batch.  For n_in <= 64 and
 * n_out <= 256 the whole forward pass is one tensor-core kernel that keeps each 128-row tile's
 * activations on chip (SiLU through a hardware tanh approximation); other shapes run layer by
 * layer. */
souffle_status souffle_mlp_forward(souffle_mlp* h, const float* x_dev, int32_t m, float* y_dev);
/* The same forward pass one GEMM per layer, activations through device memory (the path the
 * training steps use, with SiLU from an exponential and a division). */
souffle_status souffle_mlp_forward_layered(souffle_mlp* h, const float* x_dev, int32_t m, float* y_dev);

/* Benchmark utility: runs the forward pass over the m rows already in the network's input buffer
 * (the last souffle_mlp_forward call's input) iters times back to back on the network's stream,
 * fused (1) or layer by layer (0), and reports the mean device time per pass in *us (CUDA
 * events around the launches; no input packing or output unpadding). */
souffle_status souffle_mlp_profile_forward(souffle_mlp* h, int32_t m, int32_t iters, int32_t fused, double* us);

/* Loss and gradient of the loss with respect to every parameter (flat layout above, host array
 * of souffle_mlp_param_count floats) for one batch; parameters unchanged. */
souffle_status souffle_mlp_gradients(souffle_mlp* h, const float* x_dev, const float* t_dev, int32_t m,
                                     float* loss, float* grad_host);

/* One Adam step (beta1 0.9, beta2 0.999, eps 1e-8) on one batch; *loss is the batch loss before
 * the step. */
souffle_status souffle_mlp_train_step(souffle_mlp* h, const float* x_dev, const float* t_dev, int32_t m, float lr,
                                      float* loss);

/* ---- the surrogate inside a system handle ---------------------------------------------------
 * A subunit pair (A, B) is "far" when its closest bead pair is at least switch_radius apart; its
 * whole interaction (Debye-Hueckel tail; no LJ/WCA contact that far out) then comes from the
 * network instead of the pair list, as forces on A's beads.  Pairs inside the switch radius stay
 * exact.  Classification happens at every pair-list rebuild.
 *
 * Descriptor of (A, B), 64 floats in A's body frame (frame from the template's centre bead and
 * two anchor beads): relative centre of mass, its length, inverse and screened inverse, the
 * orientation quaternion of B relative to A, the relative centre of mass seen from B, the 12
 * lowest elastic-mode amplitudes of A and of B (modes of the template's spring network at its
 * rest shape), 1/kappa, epsilon, the closest bead distance; zero padding.
 * Output, 6 + 3 np floats in A's body frame: total force F and torque tau on A, and per-bead
 * residuals r_i; the force on bead i is F/np + (J^-1 tau) x d_i + r_i, d_i its position relative
 * to A's centre of mass, J = sum |d|^2 I - d d^T.
 *
 * Judge: every judge_every steps one far pair in judge_stride is re-evaluated exactly; pairs are
 * binned in four classes by closest distance (switch_radius + [0, 0.5), [0.5, 1), [1, 1.5),
 * [1.5, inf)).  For each class and system the judge estimates the class's share of the
 * system's total-force RMS relative error, sqrt(judge_stride x sum over judged pairs of
 * |network - exact|^2 / sum over the system's beads of |F|^2), pairs taken as independent; a
 * class whose estimate exceeds judge_tolerance / 2 in any system reverts to exact from the next
 * rebuild on, so the four classes together stay within judge_tolerance. */
typedef struct souffle_surrogate_options {
  double switch_radius;    /* closest bead-pair distance from which a subunit pair is far, default 3.5; at least
                              every system's LJ cut-off plus its pair-list skin (BAD_INPUT otherwise) */
  int32_t far_capacity;    /* most far pairs (0 = max(1024, 2 x subunits)); beyond it all stay exact */
  int32_t judge_every;     /* default 100 */
  int32_t judge_stride;    /* default 100 (1 % of the far pairs) */
  double judge_tolerance;  /* bound on a system's total-force RMS relative error from the network, default 1e-3 */
} souffle_surrogate_options;

typedef struct souffle_surrogate_stats {
  int32_t enabled;
  int32_t far_pairs;       /* far pairs handled by the network since the last rebuild */
  int32_t far_found;       /* far pairs found at the last rebuild (> far_pairs on overflow) */
  int32_t classes_off;     /* bit c set: class c reverted to exact */
  int64_t judged;          /* pairs re-evaluated so far */
  double last_error[4];    /* per class: the estimated share of the total-force RMS relative error at
                              the last judgement (worst system), -1 = none */
} souffle_surrogate_stats;

/* Attach a network (n_in 64, n_out 6 + 3 np, max_batch >= far_capacity) to a handle whose
 * template rest shape is rest_pos [np][3].  A network trained by souffle_surrogate_fit keeps the
 * normalisation of its training data, so it can be attached to other handles of the same
 * template and switched on there without training again. */
souffle_status souffle_surrogate_attach(souffle_gpu_system* h, souffle_mlp* net, const double* rest_pos,
                                        const souffle_surrogate_options* opt);
/* Training data at the current state (surrogate switched off): classifies the far pairs and
 * writes, for up to capacity of them, raw descriptors x_dev [.][64] and exact targets
 * t_dev [.][6 + 3 np]; *count = pairs written. */
souffle_status souffle_surrogate_collect(souffle_gpu_system* h, float* x_dev, float* t_dev, int32_t capacity,
                                         int32_t* count);
/* Normalises the data set (per-feature mean and spread, kept for inference) and trains the
 * attached network on it with Adam: epochs passes of minibatches of batch rows in a seeded
 * order.  *final_loss = mean normalised loss of the last epoch. */
souffle_status souffle_surrogate_fit(souffle_gpu_system* h, const float* x_dev, const float* t_dev, int32_t n,
                                     int32_t epochs, int32_t batch, float lr, uint64_t seed, float* final_loss);
/* Switch the trained surrogate into (1) or out of (0) the force path; takes effect from the next
 * pair-list rebuild (souffle_gpu_forces with rebuild, or the next rebuild step). */
souffle_status souffle_surrogate_enable(souffle_gpu_system* h, int32_t on);
souffle_status souffle_surrogate_get_stats(souffle_gpu_system* h, souffle_surrogate_stats* out);

/* Utility: C [m][n] FP32 = A [m][k] * B [n][k]^T with A, B given as FP32 device arrays, rounded to
 * BF16 and multiplied on the tensor cores (FP32 accumulation).  For tests of the GEMM itself. */
souffle_status souffle_gemm_bf16(const float* a_dev, const float* b_dev, int32_t m, int32_t n, int32_t k,
                                 float* c_dev, int32_t device);

#ifdef __cplusplus
}
#endif

#endif
