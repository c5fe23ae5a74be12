// FP64 reductions and point-wise maps on receiver data and kernels.
#include <cuda_runtime.h>

#include <algorithm>

#include "psv_solver.hpp"

namespace psv {
namespace {

constexpr int kReduceThreads = 256;

// Per-block partial sums of 0.5 dt (obs - syn)^2 over both components
// (src/fdModel.cpp:1128-1145), in a fixed order.
__global__ void misfit_partial(size_t n, double dt, const double *ou, const double *su,
                               const double *oz, const double *sz, double *partials) {
  __shared__ double acc[kReduceThreads];
  double s = 0;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n;
       i += (size_t)gridDim.x * blockDim.x) {
    const double a = ou[i] - su[i], b = oz[i] - sz[i];
    s += 0.5 * dt * (a * a);
    s += 0.5 * dt * (b * b);
  }
  acc[threadIdx.x] = s;
  __syncthreads();
  for (int w = kReduceThreads / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w) acc[threadIdx.x] += acc[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) partials[blockIdx.x] = acc[0];
}

__global__ void sum_partials(int n, const double *partials, double *out) {
  __shared__ double acc[kReduceThreads];
  double s = 0;
  for (int i = threadIdx.x; i < n; i += blockDim.x) s += partials[i];
  acc[threadIdx.x] = s;
  __syncthreads();
  for (int w = kReduceThreads / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w) acc[threadIdx.x] += acc[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) *out = acc[0];
}

// a = syn - obs (src/fdModel.cpp:1147-1162).
__global__ void residual(size_t n, const double *su, const double *ou, const double *sz,
                         const double *oz, double *au, double *az) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n;
       i += (size_t)gridDim.x * blockDim.x) {
    au[i] = su[i] - ou[i];
    az[i] = sz[i] - oz[i];
  }
}

// Lame -> velocity kernels with b = 1 / rho (src/fdModel.cpp:1164-1183).
__global__ void lame_to_velocity(size_t n, const double *vp, const double *vs,
                                 const double *rho, const double *kl, const double *km,
                                 const double *kr, double *kvp, double *kvs, double *krv) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n;
       i += (size_t)gridDim.x * blockDim.x) {
    const double b = 1.0 / rho[i];
    const double p = vp[i], s = vs[i], l = kl[i], m = km[i];
    kvp[i] = 2 * p * l / b;
    kvs[i] = (2 * s * m - 4 * s * l) / b;
    krv[i] = kr[i] + (p * p - 2 * s * s) * l + s * s * m;
  }
}

__global__ void reverse_residual_sum(int rows, int nt, double dt, double dxdz, const double *syn,
                                     const double *obs, double *adj) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= rows) return;
  const size_t off = (size_t)r * nt;
  double acc = 0;
  for (int n = nt - 1; n >= 0; --n) {
    acc += dt * (syn[off + n] - obs[off + n]);
    adj[off + n] = dt / dxdz * acc;
  }
}

__global__ void chain_to_velocity(size_t n, const double *vp, const double *vs, const double *rho,
                                  const double *glm, const double *gla, const double *gmu,
                                  const double *gb, double *gvp, double *gvs, double *grho) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n;
       i += (size_t)gridDim.x * blockDim.x) {
    const double p = vp[i], s = vs[i], r = rho[i];
    gvp[i] = 2.0 * r * p * (glm[i] + gla[i]);
    gvs[i] = 2.0 * r * s * gmu[i] - 4.0 * r * s * gla[i];
    grho[i] = p * p * glm[i] + (p * p - 2.0 * s * s) * gla[i] + s * s * gmu[i] - gb[i] / (r * r);
  }
}

unsigned blocks_for(size_t n) {
  size_t b = (n + 255) / 256;
  if (b > 4096) b = 4096;
  if (b == 0) b = 1;
  return static_cast<unsigned>(b);
}

}  // namespace

cudaError_t exact_receiver_terms(int rows, int nt, double dt, double dxdz, const double *syn,
                                 const double *obs, double *adj, cudaStream_t s) {
  if (rows <= 0) return cudaSuccess;
  reverse_residual_sum<<<(rows + 127) / 128, 128, 0, s>>>(rows, nt, dt, dxdz, syn, obs, adj);
  return cudaGetLastError();
}

struct StatePtrs {
  const uint4 *src[5];
  uint4 *dst[5];
  uint4 *dst2[5];
};

__global__ void copy_state_kernel(StatePtrs p, size_t n16) {
  const int f = blockIdx.y;
  const uint4 *src = p.src[f];
  uint4 *dst = p.dst[f], *dst2 = p.dst2[f];
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n16;
       i += (size_t)gridDim.x * blockDim.x) {
    const uint4 v = src[i];
    dst[i] = v;
    if (dst2) dst2[i] = v;
  }
}

cudaError_t copy_state(const void *const src[5], void *const dst[5], void *const *dst2,
                       size_t bytes, cudaStream_t s) {
  StatePtrs p;
  for (int f = 0; f < 5; ++f) {
    p.src[f] = static_cast<const uint4 *>(src[f]);
    p.dst[f] = static_cast<uint4 *>(dst[f]);
    p.dst2[f] = dst2 ? static_cast<uint4 *>(dst2[f]) : nullptr;
  }
  const size_t n16 = bytes / 16;
  if (n16 == 0) return cudaSuccess;
  const unsigned bx = static_cast<unsigned>(std::min<size_t>((n16 + 255) / 256, 1216));
  copy_state_kernel<<<dim3(bx, 5), 256, 0, s>>>(p, n16);
  return cudaGetLastError();
}

__global__ void add_into3_kernel(size_t n, const double *a0, const double *a1, const double *a2,
                                 double *b0, double *b1, double *b2) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n;
       i += (size_t)gridDim.x * blockDim.x) {
    b0[i] += a0[i];
    b1[i] += a1[i];
    b2[i] += a2[i];
  }
}

cudaError_t add_into3(size_t n, const double *const src[3], double *const dst[3], cudaStream_t s) {
  if (!n) return cudaSuccess;
  add_into3_kernel<<<blocks_for(n), 256, 0, s>>>(n, src[0], src[1], src[2], dst[0], dst[1], dst[2]);
  return cudaGetLastError();
}

cudaError_t exact_chain(size_t n, const double *vp, const double *vs, const double *rho,
                        const double *g_lm, const double *g_la, const double *g_mu,
                        const double *g_b, double *g_vp, double *g_vs, double *g_rho,
                        cudaStream_t s) {
  chain_to_velocity<<<blocks_for(n), 256, 0, s>>>(n, vp, vs, rho, g_lm, g_la, g_mu, g_b, g_vp,
                                                  g_vs, g_rho);
  return cudaGetLastError();
}

cudaError_t misfit_l2(size_t n, double dt, const double *obs_ux, const double *syn_ux,
                      const double *obs_uz, const double *syn_uz, double *partials,
                      int n_partials, double *out, cudaStream_t s) {
  misfit_partial<<<n_partials, kReduceThreads, 0, s>>>(n, dt, obs_ux, syn_ux, obs_uz, syn_uz,
                                                       partials);
  sum_partials<<<1, kReduceThreads, 0, s>>>(n_partials, partials, out);
  return cudaGetLastError();
}

cudaError_t adjoint_sources_l2(size_t n, const double *syn_ux, const double *obs_ux,
                               const double *syn_uz, const double *obs_uz, double *a_ux,
                               double *a_uz, cudaStream_t s) {
  if (!n) return cudaSuccess;
  residual<<<blocks_for(n), 256, 0, s>>>(n, syn_ux, obs_ux, syn_uz, obs_uz, a_ux, a_uz);
  return cudaGetLastError();
}

cudaError_t map_kernels(size_t n, const double *vp, const double *vs, const double *rho,
                        const double *k_lam, const double *k_mu, const double *k_rho,
                        double *vp_k, double *vs_k, double *rho_k, cudaStream_t s) {
  lame_to_velocity<<<blocks_for(n), 256, 0, s>>>(n, vp, vs, rho, k_lam, k_mu, k_rho, vp_k,
                                                 vs_k, rho_k);
  return cudaGetLastError();
}

}  // namespace psv
