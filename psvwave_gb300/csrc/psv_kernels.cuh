// P-SV velocity-stress time stepping on Virieux's staggered grid, templated
// on the wave-field precision T. Included by psv_solver_f32.cu and
// psv_solver_f64.cu only.
//
// One time step is two launches:
//   stress_step   -- records the receivers from the pre-step velocities
//                    (src/fdModel.cpp:576-596), stores the forward snapshot
//                    (src/fdModel.cpp:555-572) or correlates the adjoint field
//                    with it (src/fdModel.cpp:817-861), then advances
//                    txx, tzz, txz (src/fdModel.cpp:599-644, 864-911);
//   velocity_step -- advances vx, vz (src/fdModel.cpp:646-678, 913-948) and
//                    adds the injection terms of the point in the
//                    reference's serial order (src/fdModel.cpp:681-751,
//                    951-958).
// For T = double every expression keeps the reference's operation order;
// with contraction disabled the results are bit-identical to it.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

#include "psv_solver.hpp"

namespace psv {
namespace kern {



// Wave-field and medium arrays are stored with a row pitch (pitch >= nz,
// a multiple of 4 points so rows start on 16-byte boundaries); snapshots,
// kernels and injection cells use the reference's unpadded [nx][nz] index.
template <typename T>
struct Grid {
  int nx, nz, np, pitch;
  T dt, dx, dz;
  T *vx, *vz, *txx, *tzz, *txz;
  const T *lm, *la, *mu, *b;
  const T *taper_tab;
};

template <typename T>
__device__ __forceinline__ T taper_at(const Grid<T> &g, int ix, int iz) {
  // Number of nested absorbing frames containing the point, capped at np
  // (the counting loop of src/fdModel.cpp:273-286 in closed form).
  int c = min(min(ix + 1, iz + 1), min(g.nx - ix, g.nz - iz));
  c = min(c, g.np);
  return g.taper_tab[c];
}

// Kernel-correlation terms at one point (src/fdModel.cpp:832-858).
// a* = stored forward state, t* = current adjoint state.
template <typename T>
struct Corr;

template <>
struct Corr<double> {
  __device__ static void apply(double sidt, double lm, double la, double mu, double avx,
                               double avz, double atxx, double atzz, double atxz, double vx,
                               double vz, double txx, double tzz, double txz, double *krho,
                               double *klam, double *kmu) {
    double den = (lm - ((la * la) / (lm))) * (lm - ((la * la) / (lm)));
    *krho = *krho - sidt * (avx * vx + avz * vz);
    *klam = *klam + sidt *
                        (((atxx - (atzz * la) / lm) + (atzz - (atxx * la) / lm)) *
                         ((txx - (tzz * la) / lm) + (tzz - (txx * la) / lm))) /
                        den;
    *kmu = *kmu + sidt * 2 *
                      ((((txx - (tzz * la) / lm) * (atxx - (atzz * la) / lm)) +
                        ((tzz - (txx * la) / lm) * (atzz - (atxx * la) / lm))) /
                           den +
                       2 * (txz * atxz / (4 * mu * mu)));
  }
};

template <>
struct Corr<float> {
  // Same quantities in float arithmetic, summed into FP64 accumulators.
  __device__ static void apply(double sidt, float lm, float la, float mu, float avx, float avz,
                               float atxx, float atzz, float atxz, float vx, float vz,
                               float txx, float tzz, float txz, double *krho, double *klam,
                               double *kmu) {
    const float r = la / lm;
    const float d = lm - la * r;
    const float inv_den = 1.0f / (d * d);
    const float fxx = txx - tzz * r, fzz = tzz - txx * r;
    const float axx = atxx - atzz * r, azz = atzz - atxx * r;
    const float lam = (axx + azz) * (fxx + fzz) * inv_den;
    const float muk = (fxx * axx + fzz * azz) * inv_den + 2.0f * (txz * atxz / (4.0f * mu * mu));
    *krho = *krho - sidt * static_cast<double>(avx * vx + avz * vz);
    *klam = *klam + sidt * static_cast<double>(lam);
    *kmu = *kmu + sidt * 2.0 * static_cast<double>(muk);
  }
};

template <typename T, bool ADJ>
struct StressExtras {
  // forward: snapshot destination (null when no snapshot this step)
  T *snap[5];
  // adjoint: stored snapshot to correlate with (null when not a snapshot step)
  const T *asnap[5];
  double *krho, *klam, *kmu;
  double sidt;
  int fx0, fx1, fz0, fz1;
  // receivers (forward)
  const int *rec_cell;
  T *rec_vx, *rec_vz;  // [nr][nt]
  int nr, nt, it;
};

template <typename T, bool ADJ>
__global__ void __launch_bounds__(256) stress_step(Grid<T> g, StressExtras<T, ADJ> e) {
  const int iz = blockIdx.x * blockDim.x + threadIdx.x;
  const int ix = blockIdx.y * blockDim.y + threadIdx.y;
  if (!ADJ && e.rec_vx && blockIdx.x == 0 && blockIdx.y == 0) {
    // Pre-step receiver velocities; this launch does not modify vx, vz.
    const int tid = threadIdx.y * blockDim.x + threadIdx.x;
    for (int r = tid; r < e.nr; r += blockDim.x * blockDim.y) {
      const int c = e.rec_cell[r];
      e.rec_vx[(size_t)r * e.nt + e.it] = g.vx[c];
      e.rec_vz[(size_t)r * e.nt + e.it] = g.vz[c];
    }
  }
  if (ix >= g.nx || iz >= g.nz) return;
  const int nz = g.nz, ps = g.pitch;
  const size_t u = (size_t)ix * nz + iz;  // unpadded index
  const size_t i = (size_t)ix * ps + iz;  // padded index
  T txx = g.txx[i], tzz = g.tzz[i], txz = g.txz[i];
  if (!ADJ && e.snap[0]) {
    e.snap[0][u] = g.vx[i];
    e.snap[1][u] = g.vz[i];
    e.snap[2][u] = txx;
    e.snap[3][u] = tzz;
    e.snap[4][u] = txz;
  }
  if (ADJ && e.asnap[0] && ix >= e.fx0 && ix < e.fx1 && iz >= e.fz0 && iz < e.fz1) {
    Corr<T>::apply(e.sidt, g.lm[i], g.la[i], g.mu[i], e.asnap[0][u], e.asnap[1][u],
                   e.asnap[2][u], e.asnap[3][u], e.asnap[4][u], g.vx[i], g.vz[i], txx, tzz,
                   txz, e.krho + u, e.klam + u, e.kmu + u);
  }
  if (ix < 2 || ix >= g.nx - 2 || iz < 2 || iz >= nz - 2) return;
  const T c1 = T(9.0 / 8.0), c2 = T(1.0 / 24.0);
  const T *vx = g.vx, *vz = g.vz;
  const size_t xp1 = i + ps, xp2 = i + 2 * ps, xm1 = i - ps, xm2 = i - 2 * ps;
  const size_t zp1 = i + 1, zp2 = i + 2, zm1 = i - 1, zm2 = i - 2;
  const T lm = g.lm[i], la = g.la[i], mu = g.mu[i];
  const T tp = taper_at(g, ix, iz);
  const T dvx = c1 * (vx[xp1] - vx[i]) + c2 * (vx[xm1] - vx[xp2]);
  const T dvz = c1 * (vz[i] - vz[zm1]) + c2 * (vz[zm2] - vz[zp1]);
  const T sxx = lm * dvx / g.dx + la * dvz / g.dz;
  const T szz = la * dvx / g.dx + lm * dvz / g.dz;
  const T sxz = (c1 * (vx[zp1] - vx[i]) + c2 * (vx[zm1] - vx[zp2])) / g.dz +
                (c1 * (vz[i] - vz[xm1]) + c2 * (vz[xm2] - vz[xp1])) / g.dx;
  if (!ADJ) {
    g.txx[i] = tp * (txx + g.dt * sxx);
    g.tzz[i] = tp * (tzz + g.dt * szz);
    g.txz[i] = tp * (txz + g.dt * mu * sxz);
  } else {
    g.txx[i] = tp * (txx - g.dt * sxx);
    g.tzz[i] = tp * (tzz - g.dt * szz);
    g.txz[i] = tp * (txz - g.dt * mu * sxz);
  }
}

struct InjArgs {
  InjPlan plan;
  const double *stf;       // kind 0: [n_sources][nt]
  const double *a_ux;      // kind 1: [nr][nt] of this shot
  const double *a_uz;
  double dt;
  int nt, it;
};

template <typename T>
__device__ __forceinline__ void inject(const InjArgs &q, size_t cell, int ix, int iz, T b,
                                       T &vx, T &vz) {
  const InjPlan &p = q.plan;
  int k = p.map[(ix - p.x0) * p.h + (iz - p.z0)];
  if (k < 0) return;
  for (; k < p.n && p.terms[k].cell == (int)cell; ++k) {
    const InjTerm t = p.terms[k];
    double term;
    if (t.kind == 0) {
      term = (((t.coef * q.stf[(size_t)t.index * q.nt + q.it]) * q.dt) * (double)b) / t.div;
    } else {
      const double *a = t.field == 0 ? q.a_ux : q.a_uz;
      term = ((q.dt * (double)b) * a[(size_t)t.index * q.nt + q.it]) / t.div;
    }
    if (t.field == 0)
      vx = vx + (T)term;
    else
      vz = vz + (T)term;
  }
}

template <typename T, bool ADJ>
__global__ void __launch_bounds__(256) velocity_step(Grid<T> g, InjArgs q) {
  const int iz = blockIdx.x * blockDim.x + threadIdx.x;
  const int ix = blockIdx.y * blockDim.y + threadIdx.y;
  if (ix >= g.nx || iz >= g.nz) return;
  const int nz = g.nz, ps = g.pitch;
  const bool interior = ix >= 2 && ix < g.nx - 2 && iz >= 2 && iz < nz - 2;
  const InjPlan &p = q.plan;
  const bool in_box = p.n && ix >= p.x0 && ix < p.x0 + p.w && iz >= p.z0 && iz < p.z0 + p.h;
  if (!interior && !in_box) return;
  const size_t u = (size_t)ix * nz + iz;  // unpadded index (injection cells)
  const size_t i = (size_t)ix * ps + iz;  // padded index
  T vx = g.vx[i], vz = g.vz[i];
  const T b = g.b[i];
  if (interior) {
    const T c1 = T(9.0 / 8.0), c2 = T(1.0 / 24.0);
    const T *txx = g.txx, *tzz = g.tzz, *txz = g.txz;
    const size_t xp1 = i + ps, xp2 = i + 2 * ps, xm1 = i - ps, xm2 = i - 2 * ps;
    const size_t zp1 = i + 1, zp2 = i + 2, zm1 = i - 1, zm2 = i - 2;
    const T tp = taper_at(g, ix, iz);
    const T ax = (c1 * (txx[i] - txx[xm1]) + c2 * (txx[xm2] - txx[xp1])) / g.dx +
                 (c1 * (txz[i] - txz[zm1]) + c2 * (txz[zm2] - txz[zp1])) / g.dz;
    const T az = (c1 * (txz[xp1] - txz[i]) + c2 * (txz[xm1] - txz[xp2])) / g.dx +
                 (c1 * (tzz[zp1] - tzz[i]) + c2 * (tzz[zm1] - tzz[zp2])) / g.dz;
    if (!ADJ) {
      vx = tp * (vx + b * g.dt * ax);
      vz = tp * (vz + b * g.dt * az);
    } else {
      vx = tp * (vx - b * g.dt * ax);
      vz = tp * (vz - b * g.dt * az);
    }
  }
  if (in_box) inject<T>(q, u, ix, iz, b, vx, vz);
  g.vx[i] = vx;
  g.vz[i] = vz;
}

// rtf[r][it] = rtf[r][it-1] + dt * v / (dx * dz), serially in time per
// receiver, as src/fdModel.cpp:582-595 accumulates it.
template <typename T>
__global__ void receiver_cumsum(int nr, int nt, int n_steps, double dt, double dxdz,
                                const T *raw_x, const T *raw_z, double *rtf_x, double *rtf_z) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= 2 * nr) return;
  const int r = k >> 1;
  const T *raw = (k & 1) ? raw_z : raw_x;
  double *out = ((k & 1) ? rtf_z : rtf_x) + (size_t)r * nt;
  raw += (size_t)r * nt;
  double acc = 0;
  for (int it = 0; it < n_steps; ++it) {
    const double term = dt * (double)raw[it] / dxdz;
    acc = it == 0 ? term : acc + term;
    out[it] = acc;
  }
}

// lm = vp^2 rho, la = lm - 2 mu, mu = vs^2 rho, b = 1 / rho, computed in FP64
// (src/fdModel.cpp:1034-1051) and stored in T.
template <typename T>
__global__ void medium_kernel(int nx, int nz, int pitch, const double *vp, const double *vs,
                              const double *rho, T *lm, T *la, T *mu, T *b) {
  const int u = blockIdx.x * blockDim.x + threadIdx.x;
  if (u >= nx * nz) return;
  const int ix = u / nz, iz = u - ix * nz;
  const size_t i = (size_t)ix * pitch + iz;
  const double m = (vs[u] * vs[u]) * rho[u];
  const double l = (vp[u] * vp[u]) * rho[u];
  mu[i] = (T)m;
  lm[i] = (T)l;
  la[i] = (T)(l - 2 * m);
  b[i] = (T)(1.0 / rho[u]);
}

// dst[ix][iz] (unpadded, FP64) = src[ix * pitch + iz].
template <typename T>
__global__ void unpad_kernel(int nx, int nz, int pitch, const T *src, double *dst) {
  for (size_t u = blockIdx.x * (size_t)blockDim.x + threadIdx.x; u < (size_t)nx * nz;
       u += (size_t)gridDim.x * blockDim.x) {
    const size_t ix = u / nz, iz = u - ix * nz;
    dst[u] = (double)src[ix * pitch + iz];
  }
}

template <typename T>
__global__ void widen_kernel(size_t n, const T *src, double *dst) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n;
       i += (size_t)gridDim.x * blockDim.x)
    dst[i] = (double)src[i];
}

template <typename T>
__global__ void narrow_kernel(size_t n, const double *src, T *dst) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n;
       i += (size_t)gridDim.x * blockDim.x)
    dst[i] = (T)src[i];
}

}  // namespace kern

// ------------------------------------------------------------- drivers --

namespace kern {
// Rows of the two-kernel step's 32-column CTAs. FP64 keeps the FP64 pipe
// busy on every SM it has work on, so small CTAs spread the grid evenly over
// the SMs: at 250 x 150, 32 x 8 CTAs made 160 CTAs for 152 SMs and eight
// SMs ran two, doubling the step; one-row CTAs make 1250 (c0 FP64 gradient
// 174 ms with 32 x 8, 144 ms with 32 x 2, 141 ms with 32 x 1).
template <typename T>
struct BlockRows {
  static constexpr int value = sizeof(T) == 8 ? 1 : 8;
};
}  // namespace kern

template <typename T>
kern::Grid<T> make_grid(const SolverArgs &a) {
  kern::Grid<T> g;
  g.nx = a.nx;
  g.nz = a.nz;
  g.pitch = a.pitch;
  g.np = a.np;
  g.dt = (T)a.dt;
  g.dx = (T)a.dx;
  g.dz = (T)a.dz;
  g.vx = (T *)a.vx;
  g.vz = (T *)a.vz;
  g.txx = (T *)a.txx;
  g.tzz = (T *)a.tzz;
  g.txz = (T *)a.txz;
  g.lm = (const T *)a.lm;
  g.la = (const T *)a.la;
  g.mu = (const T *)a.mu;
  g.b = (const T *)a.b;
  g.taper_tab = (const T *)a.taper_tab;
  return g;
}

template <typename T>
cudaError_t zero_fields(const SolverArgs &a, cudaStream_t s) {
  const size_t bytes = (size_t)a.nx * a.pitch * sizeof(T);
  void *f[5] = {a.vx, a.vz, a.txx, a.tzz, a.txz};
  for (void *p : f) {
    cudaError_t e = cudaMemsetAsync(p, 0, bytes, s);
    if (e != cudaSuccess) return e;
  }
  return cudaSuccess;
}

template <typename T>
cudaError_t run_forward(const SolverArgs &a, const InjPlan &plan, int shot, bool store, int it0,
                        int it1, bool zero_first, bool finish, cudaStream_t s) {
  if (zero_first) {
    cudaError_t err = zero_fields<T>(a, s);
    if (err != cudaSuccess) return err;
  }
  const kern::Grid<T> g = make_grid<T>(a);
  const dim3 block(32, kern::BlockRows<T>::value);
  const dim3 grid((a.nz + 31) / 32, (a.nx + block.y - 1) / block.y);
  const size_t gsz = (size_t)a.nx * a.nz;
  T *raw = (T *)a.rec_raw;
  kern::StressExtras<T, false> e{};
  e.rec_cell = a.rec_cell;
  e.rec_vx = a.nr ? raw : nullptr;
  e.rec_vz = a.nr ? raw + (size_t)a.nr * a.nt : nullptr;
  e.nr = a.nr;
  e.nt = a.nt;
  kern::InjArgs q{};
  q.plan = plan;
  q.stf = a.stf;
  q.dt = a.dt;
  q.nt = a.nt;
  for (int it = it0; it < it1; ++it) {
    e.it = it;
    if (store && it % a.si == 0) {
      const size_t off = ((size_t)shot * a.snapshots + it / a.si) * gsz;
      for (int f = 0; f < 5; ++f) e.snap[f] = (T *)a.accu[f] + off;
    } else {
      for (int f = 0; f < 5; ++f) e.snap[f] = nullptr;
    }
    cudaEvent_t *ev = a.events ? a.events + 3 * (it - it0) : nullptr;
    if (ev) cudaEventRecord(ev[0], s);
    kern::stress_step<T, false><<<grid, block, 0, s>>>(g, e);
    q.it = it;
    if (ev) cudaEventRecord(ev[1], s);
    kern::velocity_step<T, false><<<grid, block, 0, s>>>(g, q);
    if (ev) cudaEventRecord(ev[2], s);
  }
  if (finish && a.nr) {
    const size_t off = (size_t)shot * a.nr * a.nt;
    if constexpr (sizeof(T) == 4)
      return receiver_cumsum_f32(a.nr, a.nt, it1, a.dt, a.dx * a.dz, (const float *)e.rec_vx,
                                 (const float *)e.rec_vz, a.rtf_ux + off, a.rtf_uz + off, s);
    else
      kern::receiver_cumsum<T><<<(2 * a.nr + 127) / 128, 128, 0, s>>>(
          a.nr, a.nt, it1, a.dt, a.dx * a.dz, e.rec_vx, e.rec_vz, a.rtf_ux + off,
          a.rtf_uz + off);
  }
  return cudaGetLastError();
}

template <typename T>
cudaError_t run_adjoint(const SolverArgs &a, const InjPlan &plan, int shot, cudaStream_t s) {
  cudaError_t err = zero_fields<T>(a, s);
  if (err != cudaSuccess) return err;
  const kern::Grid<T> g = make_grid<T>(a);
  const dim3 block(32, kern::BlockRows<T>::value);
  const dim3 grid((a.nz + 31) / 32, (a.nx + block.y - 1) / block.y);
  const size_t gsz = (size_t)a.nx * a.nz;
  kern::StressExtras<T, true> e{};
  e.krho = a.k_rho;
  e.klam = a.k_lam;
  e.kmu = a.k_mu;
  e.sidt = a.si * a.dt;
  e.fx0 = a.fx0;
  e.fx1 = a.fx1;
  e.fz0 = a.fz0;
  e.fz1 = a.fz1;
  kern::InjArgs q{};
  q.plan = plan;
  q.a_ux = a.a_stf_ux + (size_t)shot * a.nr * a.nt;
  q.a_uz = a.a_stf_uz + (size_t)shot * a.nr * a.nt;
  q.dt = a.dt;
  q.nt = a.nt;
  for (int it = a.nt - 1; it >= 0; --it) {
    if (it % a.si == 0) {
      const size_t off = ((size_t)shot * a.snapshots + it / a.si) * gsz;
      for (int f = 0; f < 5; ++f) e.asnap[f] = (const T *)a.accu[f] + off;
    } else {
      for (int f = 0; f < 5; ++f) e.asnap[f] = nullptr;
    }
    kern::stress_step<T, true><<<grid, block, 0, s>>>(g, e);
    q.it = it;
    kern::velocity_step<T, true><<<grid, block, 0, s>>>(g, q);
  }
  return cudaGetLastError();
}

template <typename T>
cudaError_t run_medium(int nx, int nz, int pitch, const double *vp, const double *vs,
                       const double *rho, void *lm, void *la, void *mu, void *b, cudaStream_t s) {
  const int n = nx * nz;
  kern::medium_kernel<T><<<(n + 255) / 256, 256, 0, s>>>(nx, nz, pitch, vp, vs, rho, (T *)lm,
                                                           (T *)la, (T *)mu, (T *)b);
  return cudaGetLastError();
}

template <typename T>
cudaError_t run_unpad(int nx, int nz, int pitch, const void *src, double *dst, cudaStream_t s) {
  size_t blocks = ((size_t)nx * nz + 255) / 256;
  if (blocks > 65535) blocks = 65535;
  if (blocks == 0) return cudaSuccess;
  kern::unpad_kernel<T><<<(unsigned)blocks, 256, 0, s>>>(nx, nz, pitch, (const T *)src, dst);
  return cudaGetLastError();
}

template <typename T>
cudaError_t run_widen(size_t n, const void *src, double *dst, cudaStream_t s) {
  if (!n) return cudaSuccess;
  size_t blocks = (n + 255) / 256;
  if (blocks > 65535) blocks = 65535;
  kern::widen_kernel<T><<<(unsigned)blocks, 256, 0, s>>>(n, (const T *)src, dst);
  return cudaGetLastError();
}

template <typename T>
cudaError_t run_narrow(size_t n, const double *src, void *dst, cudaStream_t s) {
  if (!n) return cudaSuccess;
  size_t blocks = (n + 255) / 256;
  if (blocks > 65535) blocks = 65535;
  kern::narrow_kernel<T><<<(unsigned)blocks, 256, 0, s>>>(n, src, (T *)dst);
  return cudaGetLastError();
}

}  // namespace psv

#define PSV_DEFINE_SOLVER(T, SUFFIX)                                                        \
  namespace psv {                                                                           \
  cudaError_t forward_##SUFFIX(const SolverArgs &a, const InjPlan &plan, int shot,         \
                               bool store, int it0, int it1, bool zero_first, bool finish, \
                               cudaStream_t s) {                                            \
    return run_forward<T>(a, plan, shot, store, it0, it1, zero_first, finish, s);           \
  }                                                                                         \
  cudaError_t adjoint_##SUFFIX(const SolverArgs &a, const InjPlan &plan, int shot,         \
                               cudaStream_t s) {                                            \
    return run_adjoint<T>(a, plan, shot, s);                                                \
  }                                                                                         \
  cudaError_t medium_##SUFFIX(int nx, int nz, int pitch, const double *vp, const double *vs, \
                              const double *rho, void *lm, void *la, void *mu, void *b,     \
                              cudaStream_t s) {                                             \
    return run_medium<T>(nx, nz, pitch, vp, vs, rho, lm, la, mu, b, s);                     \
  }                                                                                         \
  cudaError_t unpad_##SUFFIX(int nx, int nz, int pitch, const void *src, double *dst,       \
                             cudaStream_t s) {                                              \
    return run_unpad<T>(nx, nz, pitch, src, dst, s);                                        \
  }                                                                                         \
  cudaError_t widen_##SUFFIX(size_t n, const void *src, double *dst, cudaStream_t s) {     \
    return run_widen<T>(n, src, dst, s);                                                    \
  }                                                                                         \
  cudaError_t narrow_##SUFFIX(size_t n, const double *src, void *dst, cudaStream_t s) {    \
    return run_narrow<T>(n, src, dst, s);                                                   \
  }                                                                                         \
  }
