// Single-precision wave fields: the production path. Seismograms, misfit and
// kernel sums stay FP64.
#include "psv_exact.cuh"
#include "psv_kernels.cuh"

PSV_DEFINE_SOLVER(float, f32)
PSV_DEFINE_EXACT(float, f32)

namespace psv {
namespace kern {
// The same running sum for FP32 wave fields as a parallel FP64 prefix sum:
// one block per (receiver, component) series walks it in tiles of 256 steps
// (warp shuffles, then the 8 warp totals, then the carry from the previous
// tile). The summation order differs from the serial one by FP64 rounding
// only, far below the FP32 fields' own error; the FP64 solver keeps the
// serial receiver_cumsum for bit-exactness.
__global__ void __launch_bounds__(256) receiver_scan(int nr, int nt, int n_steps, double dt,
                                                     double dxdz, const float *raw_x,
                                                     const float *raw_z, double *rtf_x,
                                                     double *rtf_z, const int *active,
                                                     int member) {
  __shared__ double warp_total[8];
  const int k = blockIdx.x;
  if (k >= 2 * nr || (active && !active[member])) return;
  const int r = k >> 1, lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const float *raw = ((k & 1) ? raw_z : raw_x) + (size_t)r * nt;
  double *out = ((k & 1) ? rtf_z : rtf_x) + (size_t)r * nt;
  double carry = 0;
  for (int base = 0; base < n_steps; base += 256) {
    const int it = base + threadIdx.x;
    double v = it < n_steps ? dt * (double)raw[it] / dxdz : 0.0;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const double y = __shfl_up_sync(0xffffffffu, v, o);
      if (lane >= o) v += y;
    }
    if (lane == 31) warp_total[warp] = v;
    __syncthreads();
    double before = carry, tile = carry;
#pragma unroll
    for (int w = 0; w < 8; ++w) {
      const double t = warp_total[w];
      if (w < warp) before += t;
      tile += t;
    }
    if (it < n_steps) out[it] = before + v;
    __syncthreads();
    carry = tile;
  }
}

}  // namespace kern

cudaError_t receiver_cumsum_f32(int nr, int nt, int n_steps, double dt, double dxdz,
                                const float *raw_x, const float *raw_z, double *out_x,
                                double *out_z, cudaStream_t s, const int *active, int member) {
  if (nr <= 0) return cudaSuccess;
  kern::receiver_scan<<<2 * nr, 256, 0, s>>>(nr, nt, n_steps, dt, dxdz, raw_x, raw_z, out_x,
                                              out_z, active, member);
  return cudaGetLastError();
}
}  // namespace psv
