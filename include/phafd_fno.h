/*
 * Learned field propagator of the particle-field step: a spectral neural
 * operator (4 Fourier layers, channel width 32, 16 retained wavenumbers per
 * axis, GELU, BF16 weights and activations, FP32 accumulation) that, together
 * with a K-substep linearised Model-B update, advances phi over K substeps.
 * No reference counterpart: the reference advances phi only with its plain
 * Model-B update (conjugate_volfrac.cpp:89-144).  Forward and backward run on
 * the tensor cores (tcgen05) of sm_103a; training and inference act on device
 * buffers owned by the caller.
 *
 * Network.  Inputs per node: phi, bead density rho, chi (normalised with the
 * constants of phafd_fno_set_norm).  v0 = P in + pb (lift to 32 channels);
 * for l = 1..4: v_l = act(W_l v_{l-1} + b_l + S_l v_{l-1}), act = GELU for
 * l < 4, identity for l = 4; S_l is the spectral convolution with complex
 * weights R_l on the retained modes kx in [0, 8), ky, kz in [-8, 8);
 * out = q2 . GELU(Q1 v4 + q1b) + q2b; the correction is
 * out_scale * (out - mean(out)), so it carries no mass.
 *
 * Parameter vector (FP32, phafd_fno_param_count() entries, in this order):
 *   P[32][16], pb[32], then per layer W[32][32] (out, in), b[32],
 *   R[2048][32][32][2] (mode, out, in, re/im; mode = (kz' * 16 + ky') * 8 + kx),
 *   then Q1[32][32], q1b[32], q2[32], q2b.
 */
#ifndef PHAFD_FNO_H
#define PHAFD_FNO_H

#include <stddef.h>

#include "phafd_gpu.h" /* status codes PHAFD_OK, PHAFD_ERR_* */

#ifdef __cplusplus
extern "C" {
#endif

typedef struct phafd_fno phafd_fno;

/* number of FP32 parameters */
size_t phafd_fno_param_count(void);

/* network for grids of nx * ny * nz nodes (nx a multiple of 128, ny and nz
   at least 16); train != 0 allocates the activations, gradients and Adam
   state of training */
int phafd_fno_create(phafd_fno** out, int device, int nx, int ny, int nz, int train);
int phafd_fno_destroy(phafd_fno* f);
const char* phafd_fno_last_error(phafd_fno* f);

/* host FP32 parameter vector in and out */
int phafd_fno_set_params(phafd_fno* f, const float* params, size_t n);
int phafd_fno_get_params(phafd_fno* f, float* params, size_t n);

/* normalisation: phi_in = (phi - norm[0]) / norm[1]; rho_in = (rho - norm[2]) / norm[3];
   chi_in = (chi - norm[4]) / norm[5]; correction = norm[6] * (out - mean(out)) */
int phafd_fno_set_norm(phafd_fno* f, const float norm[8]);

/* correction (device, FP32, nx*ny*nz) from phi and rho (device, FP32) */
int phafd_fno_infer(phafd_fno* f, const float* phi, const float* rho, float chi, float* correction, void* stream);

/* forward + backward of loss = mean((out - target)^2) with target given in
   units of norm[6] (device, FP32); gradients are ADDED to the gradient buffer
   (phafd_fno_zero_grad clears it); loss returned on the host */
int phafd_fno_zero_grad(phafd_fno* f);
int phafd_fno_forward_backward(phafd_fno* f, const float* phi, const float* rho, float chi, const float* target,
                               double* loss);
int phafd_fno_get_grad(phafd_fno* f, float* grad, size_t n);
/* Adam step on the accumulated gradient (scaled by 1/nbatch), then zero it */
int phafd_fno_adam_step(phafd_fno* f, float lr, float beta1, float beta2, float eps, int nbatch);

/* tensor-core layout self-test: result[0] = 1 if K-major A/B products are
   exact, result[1] = 1 if the MN-major operand products are exact */
int phafd_fno_selftest(int device, int result[2]);

#ifdef __cplusplus
}
#endif

#endif
