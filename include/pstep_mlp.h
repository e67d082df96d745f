/* pstep_mlp.h -- the learned part of the particle step: a multilayer perceptron
 * that predicts a particle's self-induced disturbance of the gas at its own
 * location, trained and evaluated on the GPU by hand-written tcgen05 kernels
 * (bf16 operands, fp32 accumulation in tensor memory).
 *
 * No reference counterpart: the reference interpolates the disturbed gas state
 * (particle.cpp:340-360, 430-456) and has no correction.
 *
 * Network: PMLP_IN features -> 64 SiLU -> 64 SiLU -> PMLP_OUT outputs.
 * Parameters are one fp32 array of PMLP_NPARAM floats (the master copy; the
 * kernels round weights to bf16 for the tensor cores, biases stay fp32):
 *   W1 [64][16]  offset 0     (input columns 10..15 are padding, kept 0)
 *   b1 [64]      offset 1024
 *   W2 [64][64]  offset 1088
 *   b2 [64]      offset 5184
 *   W3 [16][64]  offset 5248  (output rows 4..15 are padding, kept 0)
 *   b3 [16]      offset 6272  (entries 4..15 padding)
 * Training minimises the mean squared error over the batch and the 4 outputs
 * with Adam (beta1 0.9, beta2 0.999, eps 1e-8), fp32 master weights.
 *
 * All functions return a pstep_status code (pstep.h). */
#ifndef PSTEP_MLP_H
#define PSTEP_MLP_H
#include <stdint.h>
#include "pstep.h"

#ifdef __cplusplus
extern "C" {
#endif

#define PMLP_IN 10
#define PMLP_HIDDEN 64
#define PMLP_OUT 4
#define PMLP_NPARAM 6288

typedef struct pmlp_ctx *pmlp_handle;

/* new network on the current CUDA device, weights drawn from `seed`
 * (uniform in +-1/sqrt(fan_in), as a default linear layer) */
int pmlp_create(uint64_t seed, pmlp_handle *out);
int pmlp_destroy(pmlp_handle h);
int pmlp_set_stream(pmlp_handle h, void *stream);

/* PMLP_NPARAM floats, host memory; set_params also clears the Adam moments */
int pmlp_get_params(pmlp_handle h, float *dst);
int pmlp_set_params(pmlp_handle h, const float *src);

/* training set: x [n][PMLP_IN] features, y [n][PMLP_OUT] targets (copied) */
int pmlp_set_data(pmlp_handle h, const float *x, const float *y, int64_t n, int on_device);

/* `steps` Adam steps on batches of `batch` rows (a multiple of 128) drawn with
 * replacement from the training set by a hash of (seed, step, slot); loss, if
 * not NULL, receives the batch loss of every step (steps floats, host) */
int pmlp_train(pmlp_handle h, int64_t steps, int batch, float lr, uint64_t seed, float *loss);

/* gradient of the mean squared error over rows [0, batch) of the training set
 * (batch a multiple of 128) at the current weights, without an update:
 * grad [PMLP_NPARAM] (host), loss (host, may be NULL) */
int pmlp_gradient(pmlp_handle h, int batch, float *grad, float *loss);

/* outputs for n feature rows: x [n][PMLP_IN] -> y [n][PMLP_OUT] */
int pmlp_forward(pmlp_handle h, const float *x, int64_t n, float *y, int on_device);

/* Adam steps taken so far */
int64_t pmlp_steps(pmlp_handle h);
/* tensor-core kernel launches made by this handle so far */
int64_t pmlp_launch_count(pmlp_handle h);
const char *pmlp_last_error(pmlp_handle h);

#ifdef __cplusplus
}
#endif
#endif
