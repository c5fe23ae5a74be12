// Exact discrete adjoint of the time step: the transpose of the forward
// update of psv_kernels.cuh, applied backwards in time, giving the gradient of
// the L2 misfit (src/fdModel.cpp:1128-1145) with respect to the medium.
//
// The reference's adjoint (src/fdModel.cpp:789-969) re-runs the forward
// scheme in reverse time with the adjoint sources injected and correlates
// snapshots; that is the continuous adjoint discretised, not the transpose
// of the discrete forward operator, and its kernels differ from finite
// differences of the discrete misfit by percents. This file is the
// transpose. Notation per step n (state x^n = (v^n, tau^n) at the start of
// step n, interior points I = [2, n-2) in both axes, T the taper):
//
//   forward:  tau' = T (tau + dt C E v)            on I, tau' = tau elsewhere
//             v'   = T (v + b dt A tau') + s^n     on I, v'   = v + s^n elsewhere
//   E v = (Dx+ vx / dx, Dz- vz / dz, Dz+ vx / dz + Dx- vz / dx)
//   A t = (Dx- txx / dx + Dz- txz / dz, Dx+ txz / dx + Dz+ tzz / dz)
//   C   = [[lm, la], [la, lm]] on (xx, zz), mu on xz
//
// with D- f(i) = c1 (f(i) - f(i-1)) + c2 (f(i-2) - f(i+1)),
//      D+ f(i) = c1 (f(i+1) - f(i)) + c2 (f(i-1) - f(i+2)),
// whose transposes (for a field g that vanishes outside I) are -D+ and -D-.
// Given the adjoint state l^{n+1} = (lv, lt):
//
//   step 1 (velocity transpose):  w = b dt T lv on I (0 elsewhere)
//          lt~ = lt + A^T w;  grad_b += dt T lv . A tau^{n+1};  source terms
//   step 2 (stress transpose):    y = T lt~ on I (0 elsewhere)
//          tau-bar^n = y on I, lt~ elsewhere
//          v-bar^n   = T lv on I (lv elsewhere) + E^T (dt C y) + receiver term
//          grad_lm += dt (y_xx ex + y_zz ez), grad_la += dt (y_xx ez + y_zz ex),
//          grad_mu += dt y_xz gxz   (strain rates of v^n)
//
// Medium gradients accumulate in FP64. Included by psv_solver_f32.cu and
// psv_solver_f64.cu.
#pragma once

#include <cuda_runtime.h>

#include "psv_solver.hpp"
#include "psv_pdl.cuh"

namespace psv {
namespace exact {

template <typename T>
struct AdjArgs {
  int nx, nz, pitch, np;
  T dt, idx, idz;  // time step, 1 / dx, 1 / dz
  const T *lm, *la, *mu, *b, *taper_tab;  // padded [nx][pitch]
  // adjoint state: velocities (updated in place by step 2), stresses in
  // (updated in place by step 1) and out (written by step 2)
  T *lvx, *lvz;
  T *ltxx, *ltzz, *ltxz;
  T *otxx, *otzz, *otxz;
  // forward states: v^n (for E) and tau^{n+1} (for A), padded
  const T *fvx, *fvz;
  const T *ftxx, *ftzz, *ftxz;
  // FP64 medium gradients, unpadded [nx][nz]
  double *g_lm, *g_la, *g_mu, *g_b;
  // scratch, padded: w = b dt T lv (step 1) and p_x, p_z, q = dt C y (step 2)
  T *wx, *wz, *px, *pz, *qq;
};

template <typename T>
__device__ __forceinline__ T taper_of(const AdjArgs<T> &a, int ix, int iz) {
  int c = min(min(ix + 1, iz + 1), min(a.nx - ix, a.nz - iz));
  return a.taper_tab[min(c, a.np)];
}

template <typename T>
__device__ __forceinline__ bool interior(const AdjArgs<T> &a, int ix, int iz) {
  return ix >= 2 && ix < a.nx - 2 && iz >= 2 && iz < a.nz - 2;
}

// w(i) = b dt T lv at interior points, 0 elsewhere (incl. outside the grid).
template <typename T>
__device__ __forceinline__ T w_at(const AdjArgs<T> &a, const T *lv, int ix, int iz) {
  if (ix < 0 || ix >= a.nx || iz < 0 || iz >= a.nz || !interior(a, ix, iz)) return T(0);
  const size_t p = (size_t)ix * a.pitch + iz;
  return a.b[p] * a.dt * taper_of(a, ix, iz) * lv[p];
}

// A padded scratch field at (x, z), 0 outside the grid (the fields hold 0
// outside the interior already).
template <typename T>
__device__ __forceinline__ T at(const AdjArgs<T> &a, const T *f, int x, int z) {
  if (x < 0 || x >= a.nx || z < 0 || z >= a.nz) return T(0);
  return f[(size_t)x * a.pitch + z];
}

// w = b dt T lv, once per point (each is used at 9 stencil points).
template <typename T>
__global__ void w_fields(AdjArgs<T> a) {
  kern::pdl_wait();
  const int iz = blockIdx.x * blockDim.x + threadIdx.x;
  const int ix = blockIdx.y * blockDim.y + threadIdx.y;
  if (ix >= a.nx || iz >= a.nz) return;
  const size_t p = (size_t)ix * a.pitch + iz;
  a.wx[p] = w_at(a, a.lvx, ix, iz);
  a.wz[p] = w_at(a, a.lvz, ix, iz);
}

// p_x, p_z, q = dt C y of the updated adjoint stresses, once per point.
template <typename T>
__device__ __forceinline__ void pq_at(const AdjArgs<T> &a, int ix, int iz, T &px, T &pz, T &q);

template <typename T>
__global__ void pq_fields(AdjArgs<T> a) {
  kern::pdl_wait();
  const int iz = blockIdx.x * blockDim.x + threadIdx.x;
  const int ix = blockIdx.y * blockDim.y + threadIdx.y;
  if (ix >= a.nx || iz >= a.nz) return;
  const size_t p = (size_t)ix * a.pitch + iz;
  T px, pz, q;
  pq_at(a, ix, iz, px, pz, q);
  a.px[p] = px;
  a.pz[p] = pz;
  a.qq[p] = q;
}

template <typename T>
__global__ void velocity_transpose(AdjArgs<T> a, InjPlan plan, const double *stf, int nt,
                                   int it, double dt_d) {
  kern::pdl_wait();
  const int iz = blockIdx.x * blockDim.x + threadIdx.x;
  const int ix = blockIdx.y * blockDim.y + threadIdx.y;
  if (ix >= a.nx || iz >= a.nz) return;
  const T c1 = T(9.0 / 8.0), c2 = T(1.0 / 24.0);
  const size_t p = (size_t)ix * a.pitch + iz;
  const size_t u = (size_t)ix * a.nz + iz;
  // A^T w with A^T = (-Dx+ on txx, -Dz- and -Dx- ... ) as in the header.
  auto wx = [&](int x, int z) { return at(a, a.wx, x, z); };
  auto wz = [&](int x, int z) { return at(a, a.wz, x, z); };
  // -D+_x(wx)(j) / dx into txx: D+ g(j) = c1 (g(j+1) - g(j)) + c2 (g(j-1) - g(j+2))
  const T dxp_wx = c1 * (wx(ix + 1, iz) - wx(ix, iz)) + c2 * (wx(ix - 1, iz) - wx(ix + 2, iz));
  const T dzp_wx = c1 * (wx(ix, iz + 1) - wx(ix, iz)) + c2 * (wx(ix, iz - 1) - wx(ix, iz + 2));
  // -D-_z(wz)(j) / dz into tzz: D- g(j) = c1 (g(j) - g(j-1)) + c2 (g(j-2) - g(j+1))
  const T dzm_wz = c1 * (wz(ix, iz) - wz(ix, iz - 1)) + c2 * (wz(ix, iz - 2) - wz(ix, iz + 1));
  const T dxm_wz = c1 * (wz(ix, iz) - wz(ix - 1, iz)) + c2 * (wz(ix - 2, iz) - wz(ix + 1, iz));
  a.ltxx[p] = a.ltxx[p] - dxp_wx * a.idx;
  a.ltzz[p] = a.ltzz[p] - dzm_wz * a.idz;
  a.ltxz[p] = a.ltxz[p] - dzp_wx * a.idz - dxm_wz * a.idx;
  if (interior(a, ix, iz)) {
    // grad_b += dt T lv . A tau^{n+1}
    const T *txx = a.ftxx, *tzz = a.ftzz, *txz = a.ftxz;
    const size_t ps = a.pitch;
    const T ax = (c1 * (txx[p] - txx[p - ps]) + c2 * (txx[p - 2 * ps] - txx[p + ps])) * a.idx +
                 (c1 * (txz[p] - txz[p - 1]) + c2 * (txz[p - 2] - txz[p + 1])) * a.idz;
    const T az = (c1 * (txz[p + ps] - txz[p]) + c2 * (txz[p - ps] - txz[p + 2 * ps])) * a.idx +
                 (c1 * (tzz[p + 1] - tzz[p]) + c2 * (tzz[p - 1] - tzz[p + 2])) * a.idz;
    const T tp = taper_of(a, ix, iz);
    a.g_b[u] += (double)(a.dt * tp) * ((double)a.lvx[p] * (double)ax + (double)a.lvz[p] * (double)az);
  }
  // Source terms s = coef stf dt b / div at their points depend on b.
  if (plan.n && ix >= plan.x0 && ix < plan.x0 + plan.w && iz >= plan.z0 && iz < plan.z0 + plan.h) {
    int k = plan.map[(ix - plan.x0) * plan.h + (iz - plan.z0)];
    for (; k >= 0 && k < plan.n && plan.terms[k].cell == (int)u; ++k) {
      const InjTerm t = plan.terms[k];
      if (t.kind != 0) continue;
      const double ds = ((t.coef * stf[(size_t)t.index * nt + it]) * dt_d) / t.div;
      a.g_b[u] += ds * (double)(t.field == 0 ? a.lvx[p] : a.lvz[p]);
    }
  }
}

template <typename T>
__device__ __forceinline__ void y_at(const AdjArgs<T> &a, int ix, int iz, T &yxx, T &yzz, T &yxz) {
  if (ix < 0 || ix >= a.nx || iz < 0 || iz >= a.nz || !interior(a, ix, iz)) {
    yxx = yzz = yxz = T(0);
    return;
  }
  const size_t p = (size_t)ix * a.pitch + iz;
  const T tp = taper_of(a, ix, iz);
  yxx = tp * a.ltxx[p];
  yzz = tp * a.ltzz[p];
  yxz = tp * a.ltxz[p];
}

// p_x = dt (lm y_xx + la y_zz), p_z = dt (la y_xx + lm y_zz), q = dt mu y_xz
template <typename T>
__device__ __forceinline__ void pq_at(const AdjArgs<T> &a, int ix, int iz, T &px, T &pz, T &q) {
  T yxx, yzz, yxz;
  y_at(a, ix, iz, yxx, yzz, yxz);
  if (yxx == T(0) && yzz == T(0) && yxz == T(0)) {
    px = pz = q = T(0);
    return;
  }
  const size_t p = (size_t)ix * a.pitch + iz;
  px = a.dt * (a.lm[p] * yxx + a.la[p] * yzz);
  pz = a.dt * (a.la[p] * yxx + a.lm[p] * yzz);
  q = a.dt * a.mu[p] * yxz;
}

template <typename T>
__global__ void stress_transpose(AdjArgs<T> a) {
  kern::pdl_wait();
  const int iz = blockIdx.x * blockDim.x + threadIdx.x;
  const int ix = blockIdx.y * blockDim.y + threadIdx.y;
  if (ix >= a.nx || iz >= a.nz) return;
  const T c1 = T(9.0 / 8.0), c2 = T(1.0 / 24.0);
  const size_t p = (size_t)ix * a.pitch + iz;
  const size_t u = (size_t)ix * a.nz + iz;
  const bool in = interior(a, ix, iz);
  const T tp = in ? taper_of(a, ix, iz) : T(1);
  // tau-bar^n
  a.otxx[p] = tp * a.ltxx[p];
  a.otzz[p] = tp * a.ltzz[p];
  a.otxz[p] = tp * a.ltxz[p];
  // E^T (dt C y):  v-bar_x += -D-_x(p_x)/dx - D-_z(q)/dz,
  //                v-bar_z += -D+_z(p_z)/dz - D+_x(q)/dx
  const T px0 = at(a, a.px, ix, iz), pz0 = at(a, a.pz, ix, iz), q0 = at(a, a.qq, ix, iz);
  const T pxm1 = at(a, a.px, ix - 1, iz), pxm2 = at(a, a.px, ix - 2, iz),
          pxp1 = at(a, a.px, ix + 1, iz);
  const T qzm1 = at(a, a.qq, ix, iz - 1), qzm2 = at(a, a.qq, ix, iz - 2),
          qzp1 = at(a, a.qq, ix, iz + 1);
  const T pzp1 = at(a, a.pz, ix, iz + 1), pzp2 = at(a, a.pz, ix, iz + 2),
          pzm1 = at(a, a.pz, ix, iz - 1);
  const T qxp1 = at(a, a.qq, ix + 1, iz), qxp2 = at(a, a.qq, ix + 2, iz),
          qxm1 = at(a, a.qq, ix - 1, iz);
  const T dxm_px = c1 * (px0 - pxm1) + c2 * (pxm2 - pxp1);
  const T dzm_q = c1 * (q0 - qzm1) + c2 * (qzm2 - qzp1);
  const T dzp_pz = c1 * (pzp1 - pz0) + c2 * (pzm1 - pzp2);
  const T dxp_q = c1 * (qxp1 - q0) + c2 * (qxm1 - qxp2);
  a.lvx[p] = tp * a.lvx[p] - dxm_px * a.idx - dzm_q * a.idz;
  a.lvz[p] = tp * a.lvz[p] - dzp_pz * a.idz - dxp_q * a.idx;
  if (in) {
    // Medium gradients from the strain rates of v^n.
    const T *vx = a.fvx, *vz = a.fvz;
    const size_t ps = a.pitch;
    const T ex = (c1 * (vx[p + ps] - vx[p]) + c2 * (vx[p - ps] - vx[p + 2 * ps])) * a.idx;
    const T ez = (c1 * (vz[p] - vz[p - 1]) + c2 * (vz[p - 2] - vz[p + 1])) * a.idz;
    const T gxz = (c1 * (vx[p + 1] - vx[p]) + c2 * (vx[p - 1] - vx[p + 2])) * a.idz +
                  (c1 * (vz[p] - vz[p - ps]) + c2 * (vz[p - 2 * ps] - vz[p + ps])) * a.idx;
    const double yxx = (double)(tp * a.ltxx[p]), yzz = (double)(tp * a.ltzz[p]),
                 yxz = (double)(tp * a.ltxz[p]);
    const double dt = (double)a.dt;
    a.g_lm[u] += dt * (yxx * (double)ex + yzz * (double)ez);
    a.g_la[u] += dt * (yxx * (double)ez + yzz * (double)ex);
    a.g_mu[u] += dt * yxz * (double)gxz;
  }
}

// Receiver term: v-bar^n(rec) += adj[r][n] (both components). One thread
// per (cell, component) adds the terms of the receivers at that cell in
// increasing receiver index, so coinciding receivers add in a fixed order
// (the same sums as one serial pass over the receivers).
template <typename T>
__global__ void add_receiver_terms(int n_groups, int nt, int it, const int *cells,
                                   const int *start, const int *order, const double *adj_x,
                                   const double *adj_z, T *lvx, T *lvz) {
  kern::pdl_wait();
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= 2 * n_groups) return;
  const int grp = k >> 1, comp = k & 1;
  T *lv = comp == 0 ? lvx : lvz;
  const double *adj = comp == 0 ? adj_x : adj_z;
  const int j0 = start[grp], j1 = start[grp + 1];
  const int c = cells[order[j0]];  // padded cell
  T v = lv[c];
  for (int j = j0; j < j1; ++j) v = v + (T)adj[(size_t)order[j] * nt + it];
  lv[c] = v;
}

}  // namespace exact

// Exact-adjoint helpers (precision-specific, defined with PSV_DEFINE_EXACT).
#define PSV_DEFINE_EXACT(T, SUFFIX)                                                           \
  namespace psv {                                                                             \
  cudaError_t exact_step_##SUFFIX(const ExactStepArgs &e, cudaStream_t s) {                  \
    exact::AdjArgs<T> a;                                                                      \
    a.nx = e.nx;                                                                              \
    a.nz = e.nz;                                                                              \
    a.pitch = e.pitch;                                                                        \
    a.np = e.np;                                                                              \
    a.dt = (T)e.dt;                                                                           \
    a.idx = (T)(1.0 / e.dx);                                                                  \
    a.idz = (T)(1.0 / e.dz);                                                                  \
    a.lm = (const T *)e.lm;                                                                   \
    a.la = (const T *)e.la;                                                                   \
    a.mu = (const T *)e.mu;                                                                   \
    a.b = (const T *)e.b;                                                                     \
    a.taper_tab = (const T *)e.taper_tab;                                                     \
    a.lvx = (T *)e.lv[0];                                                                     \
    a.lvz = (T *)e.lv[1];                                                                     \
    a.ltxx = (T *)e.lt[0];                                                                    \
    a.ltzz = (T *)e.lt[1];                                                                    \
    a.ltxz = (T *)e.lt[2];                                                                    \
    a.otxx = (T *)e.ot[0];                                                                    \
    a.otzz = (T *)e.ot[1];                                                                    \
    a.otxz = (T *)e.ot[2];                                                                    \
    a.fvx = (const T *)e.fv[0];                                                               \
    a.fvz = (const T *)e.fv[1];                                                               \
    a.ftxx = (const T *)e.ft[0];                                                              \
    a.ftzz = (const T *)e.ft[1];                                                              \
    a.ftxz = (const T *)e.ft[2];                                                              \
    a.g_lm = e.g_lm;                                                                          \
    a.g_la = e.g_la;                                                                          \
    a.g_mu = e.g_mu;                                                                          \
    a.g_b = e.g_b;                                                                            \
    a.wx = (T *)e.scratch[0];                                                                 \
    a.wz = (T *)e.scratch[1];                                                                 \
    a.px = (T *)e.scratch[2];                                                                 \
    a.pz = (T *)e.scratch[3];                                                                 \
    a.qq = (T *)e.scratch[4];                                                                 \
    const dim3 block(32, 8), grid((e.nz + 31) / 32, (e.nx + 7) / 8);                          \
    cudaError_t le = kern::launch_pdl(exact::w_fields<T>, grid, block, s, a);                   \
    if (le == cudaSuccess)                                                                    \
      le = kern::launch_pdl(exact::velocity_transpose<T>, grid, block, s, a, e.plan, e.stf,   \
                            e.nt, e.it, e.dt);                                                \
    if (le == cudaSuccess) le = kern::launch_pdl(exact::pq_fields<T>, grid, block, s, a);      \
    if (le == cudaSuccess) le = kern::launch_pdl(exact::stress_transpose<T>, grid, block, s, a); \
    if (le == cudaSuccess && e.n_rec_groups)                                                  \
      le = kern::launch_pdl(exact::add_receiver_terms<T>,                                     \
                            dim3((2 * e.n_rec_groups + 127) / 128), dim3(128), s,              \
                            e.n_rec_groups, e.nt, e.it, e.rec_cell, e.rec_start, e.rec_order, \
                            e.adj_x, e.adj_z, a.lvx, a.lvz);                                  \
    return le;                                                                                \
  }                                                                                           \
  }

}  // namespace psv
