// extern "C" boundary of the learned part (declared in
// include/psvwave_surrogate.h). Same conventions as psv_capi.cpp: C++
// exceptions become a status code plus the message psv_last_error() returns.
#include <cuda_runtime.h>

#include <new>
#include <string>

#include "../../include/psvwave_surrogate.h"
#include "psv_cnn.hpp"

namespace psv {
void set_last_error(const std::string &msg);  // psv_capi.cpp
}  // namespace psv

struct psv_coarse {
  psv::CoarseMap impl;
  template <typename... A>
  explicit psv_coarse(A &&...a) : impl(std::forward<A>(a)...) {}
};

struct psv_cnn {
  psv::cnn::Net impl;
  psv_cnn(int device, int max_batch) : impl(device, max_batch) {}
};

namespace {

template <class F>
int guarded(F &&f) {
  try {
    f();
    return PSV_OK;
  } catch (const psv::Error &e) {
    psv::set_last_error(e.what());
    return e.code;
  } catch (const std::bad_alloc &) {
    psv::set_last_error("host memory allocation failed");
    return PSV_ERR_INTERNAL;
  } catch (const std::exception &e) {
    psv::set_last_error(e.what());
    return PSV_ERR_INTERNAL;
  }
}

void need(const void *p, const char *what) {
  if (!p) throw psv::Error(PSV_ERR_INVALID_ARGUMENT, std::string(what) + " must not be NULL");
}

void check_device(int device) {
  int count = 0;
  if (cudaGetDeviceCount(&count) != cudaSuccess || count == 0) {
    cudaGetLastError();
    throw psv::Error(PSV_ERR_CUDA, "no CUDA device is available");
  }
  if (device < 0 || device >= count)
    throw psv::Error(PSV_ERR_INVALID_ARGUMENT, "CUDA device index out of range");
}

}  // namespace

extern "C" {

int psv_coarse_create(int device, int nx, int nz, int np, int ncx, int ncz, const double *mean,
                      const double *sigma, psv_coarse **out) {
  return guarded([&] {
    need(out, "out");
    need(mean, "mean");
    need(sigma, "sigma");
    *out = nullptr;
    check_device(device);
    *out = new psv_coarse(device, nx, nz, np, ncx, ncz, mean, sigma);
  });
}

int psv_coarse_destroy(psv_coarse *c) {
  return guarded([&] { delete c; });
}

int psv_coarse_to_fields(const psv_coarse *c, int batch, const float *z_dev, double *fields_dev,
                         void *stream) {
  return guarded([&] {
    need(c, "coarse map");
    need(z_dev, "z");
    need(fields_dev, "fields");
    if (batch < 0) throw psv::Error(PSV_ERR_INVALID_ARGUMENT, "batch must not be negative");
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    c->impl.to_fields(batch, z_dev, fields_dev, s);
  });
}

int psv_coarse_gradient(const psv_coarse *c, int batch, const double *gfields_dev, float *gz_dev,
                        double scale, void *stream) {
  return guarded([&] {
    need(c, "coarse map");
    need(gfields_dev, "gfields");
    need(gz_dev, "gz");
    if (batch < 0) throw psv::Error(PSV_ERR_INVALID_ARGUMENT, "batch must not be negative");
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    c->impl.gradient(batch, gfields_dev, gz_dev, scale, s);
  });
}

int psv_cnn_create(int device, int max_batch, psv_cnn **out) {
  return guarded([&] {
    need(out, "out");
    *out = nullptr;
    check_device(device);
    *out = new psv_cnn(device, max_batch);
  });
}

int psv_cnn_destroy(psv_cnn *n) {
  return guarded([&] { delete n; });
}

int psv_cnn_num_params(size_t *n) {
  return guarded([&] {
    need(n, "n");
    *n = psv::cnn::num_params();
  });
}

int psv_cnn_set_params(psv_cnn *n, const float *params) {
  return guarded([&] {
    need(n, "network");
    need(params, "params");
    n->impl.set_params(params);
  });
}

int psv_cnn_get_params(psv_cnn *n, float *params) {
  return guarded([&] {
    need(n, "network");
    need(params, "params");
    n->impl.get_params(params);
  });
}

int psv_cnn_predict(psv_cnn *n, int batch, const float *x_dev, float *misfit_dev,
                    float *grad_dev) {
  return guarded([&] {
    need(n, "network");
    need(x_dev, "x");
    need(misfit_dev, "misfit");
    need(grad_dev, "grad");
    n->impl.predict(batch, x_dev, misfit_dev, grad_dev);
  });
}

int psv_cnn_loss_grad(psv_cnn *n, int batch, const float *x_dev, const float *m_true_dev,
                      const float *g_true_dev, float w_misfit, float w_grad, double *loss,
                      float *dparams) {
  return guarded([&] {
    need(n, "network");
    need(x_dev, "x");
    need(m_true_dev, "m_true");
    need(g_true_dev, "g_true");
    const double l = n->impl.loss_grad(batch, x_dev, m_true_dev, g_true_dev, w_misfit, w_grad,
                                       dparams);
    if (loss) *loss = l;
  });
}

int psv_cnn_train_step(psv_cnn *n, int batch, const float *x_dev, const float *m_true_dev,
                       const float *g_true_dev, float w_misfit, float w_grad, float lr,
                       float beta1, float beta2, float eps, double *loss) {
  return guarded([&] {
    need(n, "network");
    need(x_dev, "x");
    need(m_true_dev, "m_true");
    need(g_true_dev, "g_true");
    psv::cnn::Adam opt;
    opt.lr = lr;
    opt.beta1 = beta1;
    opt.beta2 = beta2;
    opt.eps = eps;
    const double l = n->impl.train_step(batch, x_dev, m_true_dev, g_true_dev, w_misfit, w_grad,
                                        opt);
    if (loss) *loss = l;
  });
}

}  // extern "C"
