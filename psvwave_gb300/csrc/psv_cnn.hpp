// Surrogate network of the Monte Carlo workload: a 4-layer convolutional net
// over the coarse medium parameters (3 channels vp, vs, rho on a 20 x 10
// grid, in prior-normalised units, plus 2 channels holding each node's x and
// z coordinate, since the sensitivity of the data depends on where a node
// sits relative to sources and receivers) that predicts the L2 misfit and
// its gradient with respect to the parameters. No counterpart in the
// reference, which has no learned part.
//
//   layer 1: 3x3 conv  5 -> 32, dilation 1, ReLU
//   layer 2: 3x3 conv 32 -> 64, dilation 2, ReLU
//   layer 3: 3x3 conv 64 -> 64, dilation 4, ReLU
//   layer 4: 3x3 conv 64 ->  4, dilation 1
//   outputs: gradient map = channels 0..2; misfit = sum over the grid of
//            channel 3.
//
// Zero padding, "same" size. Weights are BF16 (an FP32 master copy is kept
// for training); activations and accumulation are FP32. Training is plain
// Adam on a weighted mean-squared error of both outputs. Every kernel is
// deterministic (fixed reduction orders, no atomics).
#pragma once

#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cstddef>

#include "psv_model.hpp"

namespace psv {
namespace cnn {

constexpr int kH = 20, kW = 10, kP = kH * kW;  // coarse grid: x rows, z columns
constexpr int kLayers = 4;
constexpr int kCin[kLayers] = {5, 32, 64, 64};
constexpr int kCout[kLayers] = {32, 64, 64, 4};
constexpr int kDil[kLayers] = {1, 2, 4, 1};
constexpr int kMaxC = 64;
constexpr int kChunks = 32;  // position ranges of the weight-gradient partial sums

// Parameter vector layout: for each layer, weights [cout][cin][3][3] then
// bias [cout].
size_t weight_offset(int layer);
size_t bias_offset(int layer);
size_t num_params();

struct Adam {
  float lr = 1e-3f, beta1 = 0.9f, beta2 = 0.999f, eps = 1e-8f;
};

class Net {
 public:
  Net(int device, int max_batch);
  ~Net();
  Net(const Net &) = delete;
  Net &operator=(const Net &) = delete;

  void set_params(const float *host);
  void get_params(float *host);
  // Inference: x [B][5][kP] -> misfit [B], gradient [B][3][kP] (device).
  void predict(int batch, const float *x, float *misfit, float *grad);
  // Loss and parameter gradient (host, num_params floats) of a batch.
  double loss_grad(int batch, const float *x, const float *m_true, const float *g_true,
                   float w_misfit, float w_grad, float *dparams_host);
  // One Adam step on a batch; returns the batch loss before the step.
  double train_step(int batch, const float *x, const float *m_true, const float *g_true,
                    float w_misfit, float w_grad, const Adam &opt);
  int device() const { return device_; }
  int max_batch() const { return max_batch_; }

 private:
  void forward(int batch, const float *x);
  double backward(int batch, const float *x, const float *m_true, const float *g_true,
                  float w_misfit, float w_grad);
  void refresh_bf16();
  void check_batch(int batch) const;

  int device_, max_batch_;
  cudaStream_t stream_ = nullptr;
  int step_ = 0;
  DeviceBuffer params_, wbf_, grads_, partials_, adam_m_, adam_v_;
  DeviceBuffer act_[kLayers];   // layer outputs [B][cout][kP] (post-ReLU for 1..3)
  DeviceBuffer dact_[2];        // gradient scratch [B][kMaxC][kP]
  DeviceBuffer loss_partials_, loss_;
  DeviceBuffer err_;  // int, raised by a tensor-core convolution's bounded wait
  void check_error();
};

}  // namespace cnn

// Coarse-to-grid map of the Monte Carlo workload: medium parameters on an
// ncx x ncz grid over the inner region, theta = mean + sigma * z per
// channel (vp, vs, rho), bilinearly interpolated to the inner grid (node
// (i, j) at fine inner position ((i + 0.5) fx - 0.5, (j + 0.5) fz - 0.5),
// clamped at the ends) and replicated outward into the absorbing boundary.
class CoarseMap {
 public:
  CoarseMap(int device, int nx, int nz, int np, int ncx, int ncz, const double *mean,
            const double *sigma);
  ~CoarseMap();
  CoarseMap(const CoarseMap &) = delete;
  CoarseMap &operator=(const CoarseMap &) = delete;
  // z [B][3][ncx][ncz] (FP32, device) -> fields [B][3][nx][nz] (FP64, device),
  // on stream s, or synchronously on the map's own stream when s is null.
  void to_fields(int batch, const float *z, double *fields, cudaStream_t s) const;
  // Transpose: field gradients [B][3][nx][nz] -> z gradients [B][3][ncx][ncz],
  // scaled by `scale`; streams as to_fields.
  void gradient(int batch, const double *gfields, float *gz, double scale, cudaStream_t s) const;
  int nx, nz, np, ncx, ncz;

 private:
  int device_;
  cudaStream_t stream_ = nullptr;  // non-blocking; used when the caller passes none
  DeviceBuffer x0_, x1_, wx_, z0_, z1_, wz_;   // per fine index
  DeviceBuffer xs_, xe_, zs_, ze_;             // per coarse index: fine support
  DeviceBuffer mean_, sigma_;
};

}  // namespace psv
