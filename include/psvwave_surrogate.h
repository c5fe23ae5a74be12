/*
 * psvwave_surrogate.h -- C ABI of the learned part of psvwave_gb300: the
 * surrogate network and the coarse medium parameterisation of the
 * surrogate-screened Monte Carlo workload.
 *
 * None of these entry points has a counterpart in the reference
 * (larsgeb/psvWave), which is a plain finite-difference library. The
 * conventions are those of psvwave.h: an int status (PSV_OK or PSV_ERR_*),
 * the message in psv_last_error(), no exceptions across the boundary.
 * Buffers named *_dev are device pointers on the object's device; the calls
 * synchronise before returning unless a stream is passed.
 */
#ifndef PSVWAVE_SURROGATE_H
#define PSVWAVE_SURROGATE_H

#include <stddef.h>

#include "psvwave.h"

#ifdef __cplusplus
extern "C" {
#endif

/* ---- coarse parameterisation --------------------------------------------
 * The medium (vp, vs, rho) on an ncx x ncz grid over the inner region:
 * theta = mean + sigma * z per channel, bilinearly interpolated to the inner
 * grid (node (i, j) at fine inner position ((i + 0.5) fx - 0.5,
 * (j + 0.5) fz - 0.5) with fx = nx_inner / ncx, clamped at the ends) and
 * replicated outward into the np-frame absorbing boundary. */
typedef struct psv_coarse psv_coarse;
/* mean, sigma: host [3][ncx][ncz]. */
int psv_coarse_create(int device, int nx, int nz, int np, int ncx, int ncz, const double *mean,
                      const double *sigma, psv_coarse **out);
int psv_coarse_destroy(psv_coarse *c);
/* z_dev [batch][3][ncx][ncz] (float) -> fields_dev [batch][3][nx][nz]
 * (double: vp, vs, rho grids in the layout psv_set_parameter_fields_device
 * takes). stream: a cudaStream_t, or NULL for a synchronous call. */
int psv_coarse_to_fields(const psv_coarse *c, int batch, const float *z_dev, double *fields_dev,
                         void *stream);
/* Transpose of the map times `scale`: gradients with respect to the three
 * fields gfields_dev [batch][3][nx][nz] -> gradients with respect to z,
 * gz_dev [batch][3][ncx][ncz]. */
int psv_coarse_gradient(const psv_coarse *c, int batch, const double *gfields_dev, float *gz_dev,
                        double scale, void *stream);

/* ---- surrogate network ---------------------------------------------------
 * 4 layers of 3x3 convolutions over [5][20][10] inputs -- the 3 parameter
 * channels and 2 channels of node coordinates -- (channels 5-32-64-64-4,
 * dilations 1, 2, 4, 1, ReLU between layers), BF16 weights with an FP32
 * master copy, FP32 activations and accumulation. Outputs: the predicted
 * misfit (sum over the grid of channel 3) and gradient map (channels 0..2).
 * Parameter vector: per layer, weights [cout][cin][3][3] then bias [cout]. */
typedef struct psv_cnn psv_cnn;
int psv_cnn_create(int device, int max_batch, psv_cnn **out);
int psv_cnn_destroy(psv_cnn *n);
int psv_cnn_num_params(size_t *n);
/* Host FP32 parameter vectors; set also resets the optimiser state. */
int psv_cnn_set_params(psv_cnn *n, const float *params);
int psv_cnn_get_params(psv_cnn *n, float *params);
/* x_dev [batch][5][200] -> misfit_dev [batch], grad_dev [batch][3][200]. */
int psv_cnn_predict(psv_cnn *n, int batch, const float *x_dev, float *misfit_dev,
                    float *grad_dev);
/* Loss = w_misfit mean_b (m - m_true)^2 + w_grad mean (g - g_true)^2 of a
 * batch, and its gradient with respect to the parameters (host,
 * psv_cnn_num_params floats; NULL to skip). */
int psv_cnn_loss_grad(psv_cnn *n, int batch, const float *x_dev, const float *m_true_dev,
                      const float *g_true_dev, float w_misfit, float w_grad, double *loss,
                      float *dparams);
/* One Adam step (lr, beta1, beta2, eps) on a batch; *loss (if non-NULL) is
 * the batch loss before the step. */
int psv_cnn_train_step(psv_cnn *n, int batch, const float *x_dev, const float *m_true_dev,
                       const float *g_true_dev, float w_misfit, float w_grad, float lr,
                       float beta1, float beta2, float eps, double *loss);

#ifdef __cplusplus
}
#endif

#endif /* PSVWAVE_SURROGATE_H */
