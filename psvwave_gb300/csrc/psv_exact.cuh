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
// Both steps run in one tiled kernel. v-bar^n at a point needs dt C y at
// distance 2 (a cross), and lt~ there needs w at distance 2 again, so a tile
// of TX x TZ output points holds w over the tile grown by 4 on each side and
// p = dt C y over the tile grown by 2, both in shared memory; each CTA
// recomputes its halo of lt~ and p instead of exchanging it. lt is read only
// and the adjoint velocities go to a second buffer (the halos of the
// neighbouring tiles still read the old ones), so nothing is updated in place.
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
  // adjoint state in (lv, lt: l^{n+1}) and out (olv, olt: l^n), padded
  const T *lvx, *lvz;
  const T *ltxx, *ltzz, *ltxz;
  T *olvx, *olvz;
  T *otxx, *otzz, *otxz;
  // forward states: v^n (for E) and tau^{n+1} (for A), padded
  const T *fvx, *fvz;
  const T *ftxx, *ftzz, *ftxz;
  // FP64 medium gradients, unpadded [nx][nz]
  double *g_lm, *g_la, *g_mu, *g_b;
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

// Tile of the exact step: TX rows (x) by 32 columns (z, one warp wide),
// 256 threads.
template <typename T>
struct ExactTile;
template <>
struct ExactTile<float> {
  static constexpr int TX = 32;
};
template <>
struct ExactTile<double> {
  static constexpr int TX = 16;
};
constexpr int kExactTZ = 32;
constexpr int kExactThreads = 256;

// One exact adjoint step over a TX x 32 tile (x0 = blockIdx.y TX,
// z0 = blockIdx.x 32). Phase 1: w = b dt T lv over the tile + 4. Phase 2:
// lt~ = lt + A^T w and p = dt C y over the tile + 2 (lt~ kept for the
// tile's own points). Phase 3, per output point: tau-bar^n, the medium
// gradients, v-bar^n = T lv + E^T p, grad_b and the source terms.
template <typename T>
__global__ void __launch_bounds__(kExactThreads)
    exact_step_tile(AdjArgs<T> a, InjPlan plan, const double *stf, int nt, int it, double dt_d) {
  constexpr int TX = ExactTile<T>::TX, TZ = kExactTZ;
  constexpr int WX = TX + 8, WZ = TZ + 8;  // w region
  constexpr int PX = TX + 4, PZ = TZ + 4;  // p region
  __shared__ T sw[2][WX][WZ];
  __shared__ T sp[3][PX][PZ];
  __shared__ T slt[3][TX][TZ];
  const int x0 = blockIdx.y * TX, z0 = blockIdx.x * TZ;
  const int tid = threadIdx.x;
  const T c1 = T(9.0 / 8.0), c2 = T(1.0 / 24.0);
  kern::pdl_wait();

  // Phase 1: w(i) = b dt T lv at interior points, 0 elsewhere (incl. outside
  // the grid).
  for (int k = tid; k < WX * WZ; k += kExactThreads) {
    const int r = k / WZ, c = k - r * WZ;
    const int ix = x0 - 4 + r, iz = z0 - 4 + c;
    T wx = T(0), wz = T(0);
    if (ix >= 0 && ix < a.nx && iz >= 0 && iz < a.nz && interior(a, ix, iz)) {
      const size_t p = (size_t)ix * a.pitch + iz;
      const T s = a.b[p] * a.dt * taper_of(a, ix, iz);
      wx = s * a.lvx[p];
      wz = s * a.lvz[p];
    }
    sw[0][r][c] = wx;
    sw[1][r][c] = wz;
  }
  __syncthreads();

  // Phase 2: lt~ and p_x = dt (lm y_xx + la y_zz), p_z = dt (la y_xx + lm y_zz),
  // q = dt mu y_xz, with y = T lt~ on I and 0 elsewhere.
  for (int k = tid; k < PX * PZ; k += kExactThreads) {
    const int r = k / PZ, c = k - r * PZ;
    const int ix = x0 - 2 + r, iz = z0 - 2 + c;
    T px = T(0), pz = T(0), q = T(0);
    if (ix >= 0 && ix < a.nx && iz >= 0 && iz < a.nz) {
      const size_t p = (size_t)ix * a.pitch + iz;
      // A^T w: -D+_x(wx)/dx into txx, -D-_z(wz)/dz into tzz,
      // -D+_z(wx)/dz - D-_x(wz)/dx into txz. (r + 2, c + 2) is (ix, iz) in sw.
      const int R = r + 2, Cc = c + 2;
      const T dxp_wx = c1 * (sw[0][R + 1][Cc] - sw[0][R][Cc]) +
                       c2 * (sw[0][R - 1][Cc] - sw[0][R + 2][Cc]);
      const T dzp_wx = c1 * (sw[0][R][Cc + 1] - sw[0][R][Cc]) +
                       c2 * (sw[0][R][Cc - 1] - sw[0][R][Cc + 2]);
      const T dzm_wz = c1 * (sw[1][R][Cc] - sw[1][R][Cc - 1]) +
                       c2 * (sw[1][R][Cc - 2] - sw[1][R][Cc + 1]);
      const T dxm_wz = c1 * (sw[1][R][Cc] - sw[1][R - 1][Cc]) +
                       c2 * (sw[1][R - 2][Cc] - sw[1][R + 1][Cc]);
      const T lxx = a.ltxx[p] - dxp_wx * a.idx;
      const T lzz = a.ltzz[p] - dzm_wz * a.idz;
      const T lxz = a.ltxz[p] - dzp_wx * a.idz - dxm_wz * a.idx;
      if (r >= 2 && r < TX + 2 && c >= 2 && c < TZ + 2) {
        slt[0][r - 2][c - 2] = lxx;
        slt[1][r - 2][c - 2] = lzz;
        slt[2][r - 2][c - 2] = lxz;
      }
      if (interior(a, ix, iz)) {
        const T tp = taper_of(a, ix, iz);
        const T yxx = tp * lxx, yzz = tp * lzz, yxz = tp * lxz;
        if (!(yxx == T(0) && yzz == T(0) && yxz == T(0))) {
          px = a.dt * (a.lm[p] * yxx + a.la[p] * yzz);
          pz = a.dt * (a.la[p] * yxx + a.lm[p] * yzz);
          q = a.dt * a.mu[p] * yxz;
        }
      }
    }
    sp[0][r][c] = px;
    sp[1][r][c] = pz;
    sp[2][r][c] = q;
  }
  __syncthreads();

  // Phase 3: the tile's own points, one column per lane.
  const int c = tid % TZ;
  const int iz = z0 + c;
  if (iz >= a.nz) return;
  const size_t ps = a.pitch;
  for (int r = tid / TZ; r < TX; r += kExactThreads / TZ) {
    const int ix = x0 + r;
    if (ix >= a.nx) break;
    const size_t p = (size_t)ix * a.pitch + iz;
    const size_t u = (size_t)ix * a.nz + iz;
    const bool in = interior(a, ix, iz);
    const T tp = in ? taper_of(a, ix, iz) : T(1);
    const T lxx = slt[0][r][c], lzz = slt[1][r][c], lxz = slt[2][r][c];
    // tau-bar^n
    a.otxx[p] = tp * lxx;
    a.otzz[p] = tp * lzz;
    a.otxz[p] = tp * lxz;
    // E^T (dt C y):  v-bar_x += -D-_x(p_x)/dx - D-_z(q)/dz,
    //                v-bar_z += -D+_z(p_z)/dz - D+_x(q)/dx
    const int R = r + 2, Cc = c + 2;  // (ix, iz) in sp
    const T dxm_px = c1 * (sp[0][R][Cc] - sp[0][R - 1][Cc]) +
                     c2 * (sp[0][R - 2][Cc] - sp[0][R + 1][Cc]);
    const T dzm_q = c1 * (sp[2][R][Cc] - sp[2][R][Cc - 1]) +
                    c2 * (sp[2][R][Cc - 2] - sp[2][R][Cc + 1]);
    const T dzp_pz = c1 * (sp[1][R][Cc + 1] - sp[1][R][Cc]) +
                     c2 * (sp[1][R][Cc - 1] - sp[1][R][Cc + 2]);
    const T dxp_q = c1 * (sp[2][R + 1][Cc] - sp[2][R][Cc]) +
                    c2 * (sp[2][R - 1][Cc] - sp[2][R + 2][Cc]);
    const T lvx = a.lvx[p], lvz = a.lvz[p];
    a.olvx[p] = tp * lvx - dxm_px * a.idx - dzm_q * a.idz;
    a.olvz[p] = tp * lvz - dzp_pz * a.idz - dxp_q * a.idx;
    if (in) {
      // grad_b += dt T lv . A tau^{n+1}
      const T *txx = a.ftxx, *tzz = a.ftzz, *txz = a.ftxz;
      const T ax = (c1 * (txx[p] - txx[p - ps]) + c2 * (txx[p - 2 * ps] - txx[p + ps])) * a.idx +
                   (c1 * (txz[p] - txz[p - 1]) + c2 * (txz[p - 2] - txz[p + 1])) * a.idz;
      const T az = (c1 * (txz[p + ps] - txz[p]) + c2 * (txz[p - ps] - txz[p + 2 * ps])) * a.idx +
                   (c1 * (tzz[p + 1] - tzz[p]) + c2 * (tzz[p - 1] - tzz[p + 2])) * a.idz;
      a.g_b[u] += (double)(a.dt * tp) * ((double)lvx * (double)ax + (double)lvz * (double)az);
      // Medium gradients from the strain rates of v^n.
      const T *vx = a.fvx, *vz = a.fvz;
      const T ex = (c1 * (vx[p + ps] - vx[p]) + c2 * (vx[p - ps] - vx[p + 2 * ps])) * a.idx;
      const T ez = (c1 * (vz[p] - vz[p - 1]) + c2 * (vz[p - 2] - vz[p + 1])) * a.idz;
      const T gxz = (c1 * (vx[p + 1] - vx[p]) + c2 * (vx[p - 1] - vx[p + 2])) * a.idz +
                    (c1 * (vz[p] - vz[p - ps]) + c2 * (vz[p - 2 * ps] - vz[p + ps])) * a.idx;
      const double yxx = (double)(tp * lxx), yzz = (double)(tp * lzz), yxz = (double)(tp * lxz);
      const double dt = (double)a.dt;
      a.g_lm[u] += dt * (yxx * (double)ex + yzz * (double)ez);
      a.g_la[u] += dt * (yxx * (double)ez + yzz * (double)ex);
      a.g_mu[u] += dt * yxz * (double)gxz;
    }
    // Source terms s = coef stf dt b / div at their points depend on b.
    if (plan.n && ix >= plan.x0 && ix < plan.x0 + plan.w && iz >= plan.z0 &&
        iz < plan.z0 + plan.h) {
      int k = plan.map[(ix - plan.x0) * plan.h + (iz - plan.z0)];
      for (; k >= 0 && k < plan.n && plan.terms[k].cell == (int)u; ++k) {
        const InjTerm t = plan.terms[k];
        if (t.kind != 0) continue;
        const double ds = ((t.coef * stf[(size_t)t.index * nt + it]) * dt_d) / t.div;
        a.g_b[u] += ds * (double)(t.field == 0 ? lvx : lvz);
      }
    }
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
    a.lvx = (const T *)e.lv[0];                                                               \
    a.lvz = (const T *)e.lv[1];                                                               \
    a.ltxx = (const T *)e.lt[0];                                                              \
    a.ltzz = (const T *)e.lt[1];                                                              \
    a.ltxz = (const T *)e.lt[2];                                                              \
    a.olvx = (T *)e.ov[0];                                                                    \
    a.olvz = (T *)e.ov[1];                                                                    \
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
    const dim3 grid((e.nz + exact::kExactTZ - 1) / exact::kExactTZ,                           \
                    (e.nx + exact::ExactTile<T>::TX - 1) / exact::ExactTile<T>::TX);          \
    cudaError_t le = kern::launch_pdl(exact::exact_step_tile<T>, grid,                        \
                                      dim3(exact::kExactThreads), s, a, e.plan, e.stf, e.nt,  \
                                      e.it, e.dt);                                            \
    if (le == cudaSuccess && e.n_rec_groups)                                                  \
      le = kern::launch_pdl(exact::add_receiver_terms<T>,                                     \
                            dim3((2 * e.n_rec_groups + 127) / 128), dim3(128), s,              \
                            e.n_rec_groups, e.nt, e.it, e.rec_cell, e.rec_start, e.rec_order, \
                            e.adj_x, e.adj_z, a.olvx, a.olvz);                                \
    return le;                                                                                \
  }                                                                                           \
  }

}  // namespace psv
