// Single-precision wave fields: the production path. Seismograms, misfit and
// kernel sums stay FP64.
#include "psv_exact.cuh"
#include "psv_kernels.cuh"

PSV_DEFINE_SOLVER(float, f32)
PSV_DEFINE_EXACT(float, f32)

namespace psv {
cudaError_t receiver_cumsum_f32(int nr, int nt, int n_steps, double dt, double dxdz,
                                const float *raw_x, const float *raw_z, double *out_x,
                                double *out_z, cudaStream_t s) {
  if (nr <= 0) return cudaSuccess;
  kern::receiver_cumsum<float><<<(2 * nr + 127) / 128, 128, 0, s>>>(nr, nt, n_steps, dt, dxdz,
                                                                     raw_x, raw_z, out_x, out_z);
  return cudaGetLastError();
}
}  // namespace psv
