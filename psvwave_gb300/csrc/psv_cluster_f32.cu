// FP32 time stepping of a small grid resident in one thread-block cluster.
//
// CTA k of an nc-CTA cluster owns grid rows [x0, x0 + rows) with
// x0 = floor(k nx / nc). Its shared memory holds
//   F[5][R + 4][S]  vx, vz, txx, tzz, txz; local row lr is grid row
//                   x0 - 2 + lr, own rows lr in [2, rows + 2), halo rows 0,
//                   1 and rows + 2, rows + 3 (zero outside the grid);
//   LM, MU, B[R][S] lm, mu and b of the own rows;
//   TAP[np + 1]     the Cerjan taper by frame count;
// where R = ceil(nx / nc) and S = nz rounded up to 4 columns. One time step:
//   receivers (forward; pre-step velocities) and snapshot store (forward)
//   or correlation (adjoint) at snapshot steps;
//   stress update of the own rows; each thread that computes a point of
//     the first or last two own rows also writes its txx and txz into the
//     neighbour's halo rows (distributed shared memory);
//   cluster barrier;
//   velocity update and injection of the own rows, with the same writes of
//     vx and vz into the neighbours' halos;
//   cluster barrier.
// A halo row is written only between the barriers that bracket the
// neighbour's phase that does not read it, so two barriers per step order
// all reads and writes. The point arithmetic is the general path of
// tma::step_body (psv_tma_f32.cu) term for term, with the shared helpers
// correlate() and inject() (psv_tma_terms.cuh). Every CTA runs the same
// number of barriers, and nothing else waits.
#include <cooperative_groups.h>

#include <algorithm>

#include "psv_cluster.hpp"
#include "psv_tma_terms.cuh"

namespace psv {
namespace cluster {
namespace cg = cooperative_groups;

namespace {

constexpr int NT = 512;
constexpr int WARPS = NT / 32;

__host__ __device__ __forceinline__ int row0(int k, int nc, int nx) {
  return (int)(((long long)k * nx) / nc);
}

__host__ __device__ __forceinline__ int max_rows(int nc, int nx) { return (nx + nc - 1) / nc; }

__host__ __device__ __forceinline__ int stride(int nz) { return (nz + 3) / 4 * 4; }

size_t smem_bytes(int R, int S, int np) {
  return ((size_t)(5 * (R + 4) + 3 * R) * S + (size_t)(np + 1)) * sizeof(float);
}

// The time loop of one simulation in the calling cluster (every CTA of the
// cluster calls it with the same arguments).
template <bool ADJ>
__device__ __forceinline__ void member_steps(const tma::SimDesc &d, int nc, int it0, int n_steps,
                                             int parity, int store) {
  cg::cluster_group cl = cg::this_cluster();
  const int k = (int)cl.block_rank();
  const int nx = d.nx, nz = d.nz, ps = d.pitch, np = d.np;
  const int R = max_rows(nc, nx), S = stride(nz), FR = R + 4;
  const int x0 = row0(k, nc, nx), rows = row0(k + 1, nc, nx) - x0;
  extern __shared__ float sm[];
  float *F[5];
  for (int f = 0; f < 5; ++f) F[f] = sm + (size_t)f * FR * S;
  float *LM = sm + (size_t)5 * FR * S, *MU = LM + (size_t)R * S, *BB = MU + (size_t)R * S;
  float *TAP = BB + (size_t)R * S;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;

  // Initial state (zero outside the grid and in unused rows), medium, taper.
  {
    const fast::Fields in = d.set[parity];
    const float *src[5] = {in.vx, in.vz, in.txx, in.tzz, in.txz};
    for (int lr = warp; lr < FR; lr += WARPS) {
      const int x = x0 - 2 + lr;
      const bool row_ok = lr < rows + 4 && x >= 0 && x < nx;
      for (int z = lane; z < S; z += 32) {
        const bool ok = row_ok && z < nz;
        const size_t g = (size_t)x * ps + z;
        for (int f = 0; f < 5; ++f) F[f][lr * S + z] = ok ? src[f][g] : 0.f;
      }
    }
    for (int r = warp; r < R; r += WARPS) {
      const int x = x0 + r;
      for (int z = lane; z < S; z += 32) {
        const bool ok = r < rows && z < nz;
        const size_t g = (size_t)x * ps + z;
        LM[r * S + z] = ok ? d.lm[g] : 0.f;
        MU[r * S + z] = ok ? d.mu[g] : 0.f;
        BB[r * S + z] = ok ? d.b[g] : 0.f;
      }
    }
    for (int i = tid; i <= np; i += NT) TAP[i] = d.taper_tab[i];
  }
  // Neighbours' field arrays (distributed shared memory): rank k - 1 holds
  // rows below x0 (my rows x0, x0 + 1 are its halo rows rows_up + 2, + 3),
  // rank k + 1 rows from x0 + rows (my last two rows are its halo rows 0, 1).
  const int rows_up = k > 0 ? x0 - row0(k - 1, nc, nx) : 0;
  float *up[5], *dn[5];
  for (int f = 0; f < 5; ++f) {
    up[f] = k > 0 ? cl.map_shared_rank(F[f], k - 1) : nullptr;
    dn[f] = k + 1 < nc ? cl.map_shared_rank(F[f], k + 1) : nullptr;
  }
  cl.sync();

  const float c1 = 9.0f / 8.0f, c2 = 1.0f / 24.0f;
  const float dtv = ADJ ? -d.dt : d.dt;
  const float idx = d.idx, idz = d.idz;
  const InjPlan &pl = d.plan;
  float *const VX = F[0], *const VZ = F[1], *const TXX = F[2], *const TZZ = F[3],
              *const TXZ = F[4];

  for (int j = 0; j < n_steps; ++j) {
    const int it = ADJ ? it0 - j : it0 + j;
    const bool snap_io = (it % d.si) == 0 && d.accu[0] != nullptr && (ADJ || store);
    const size_t soff = (size_t)(it / d.si) * nx * nz;
    // Receivers: pre-step velocities at their cells.
    if (!ADJ && d.nr) {
      for (int r = tid; r < d.nr; r += NT) {
        const int c = d.rec_cell[r];
        const int ix = c / ps, iz = c - ix * ps;
        if (ix >= x0 && ix < x0 + rows) {
          d.rec_vx[(size_t)r * d.nt + it] = VX[(ix - x0 + 2) * S + iz];
          d.rec_vz[(size_t)r * d.nt + it] = VZ[(ix - x0 + 2) * S + iz];
        }
      }
    }
    // Stresses of the own rows.
    for (int lr = 2 + warp; lr < rows + 2; lr += WARPS) {
      const int gx = x0 - 2 + lr, mr = lr - 2;
      const bool x_int = gx >= 2 && gx < nx - 2;
      const bool x_free = gx >= d.fx0 && gx < d.fx1;
      // Edge rows go to the neighbours' halos (a CTA of 2 or 3 rows sends
      // a row both ways).
      const int ru = (k > 0 && lr < 4) ? (rows_up + lr) * S : -1;
      const int rd = (k + 1 < nc && lr >= rows) ? (lr - rows) * S : -1;
      for (int gz = lane; gz < nz; gz += 32) {
        const int p = lr * S + gz;
        const int g = gx * nz + gz;
        float sxx = TXX[p], szz = TZZ[p], sxz = TXZ[p];
        if (!ADJ && snap_io) {
          d.accu[0][soff + g] = VX[p];
          d.accu[1][soff + g] = VZ[p];
          d.accu[2][soff + g] = sxx;
          d.accu[3][soff + g] = szz;
          d.accu[4][soff + g] = sxz;
        }
        const float lm = LM[mr * S + gz], mu = MU[mr * S + gz];
        if (ADJ && snap_io && x_free && gz >= d.fz0 && gz < d.fz1) {
          const float *asnap[5] = {d.accu[0] + soff, d.accu[1] + soff, d.accu[2] + soff,
                                   d.accu[3] + soff, d.accu[4] + soff};
          tma::correlate(d, asnap, g, lm, mu, VX[p], VZ[p], sxx, szz, sxz);
        }
        if (x_int && gz >= 2 && gz < nz - 2) {
          const float la = lm - 2.0f * mu;
          const float dvx = c1 * (VX[p + S] - VX[p]) + c2 * (VX[p - S] - VX[p + 2 * S]);
          const float dvz = c1 * (VZ[p] - VZ[p - 1]) + c2 * (VZ[p - 2] - VZ[p + 1]);
          const float gxz = (c1 * (VX[p + 1] - VX[p]) + c2 * (VX[p - 1] - VX[p + 2])) * idz +
                            (c1 * (VZ[p] - VZ[p - S]) + c2 * (VZ[p - 2 * S] - VZ[p + S])) * idx;
          const float ex = dvx * idx, ez = dvz * idz;
          const int cnt = min(min(gz + 1, nz - gz), min(gx + 1, nx - gx));
          const float tp = cnt < np ? TAP[cnt] : 1.0f;
          sxx = tp * (sxx + dtv * (lm * ex + la * ez));
          szz = tp * (szz + dtv * (la * ex + lm * ez));
          sxz = tp * (sxz + dtv * mu * gxz);
          TXX[p] = sxx;
          TZZ[p] = szz;
          TXZ[p] = sxz;
        }
        if (ru >= 0) {
          up[2][ru + gz] = sxx;
          up[4][ru + gz] = sxz;
        }
        if (rd >= 0) {
          dn[2][rd + gz] = sxx;
          dn[4][rd + gz] = sxz;
        }
      }
    }
    cl.sync();
    // Velocities of the own rows, then injection.
    for (int lr = 2 + warp; lr < rows + 2; lr += WARPS) {
      const int gx = x0 - 2 + lr, mr = lr - 2;
      const bool x_int = gx >= 2 && gx < nx - 2;
      const bool x_box = pl.n && gx >= pl.x0 && gx < pl.x0 + pl.w;
      const int ru = (k > 0 && lr < 4) ? (rows_up + lr) * S : -1;
      const int rd = (k + 1 < nc && lr >= rows) ? (lr - rows) * S : -1;
      for (int gz = lane; gz < nz; gz += 32) {
        const int p = lr * S + gz;
        float vx = VX[p], vz = VZ[p];
        const float b = BB[mr * S + gz];
        if (x_int && gz >= 2 && gz < nz - 2) {
          const float ax = (c1 * (TXX[p] - TXX[p - S]) + c2 * (TXX[p - 2 * S] - TXX[p + S])) * idx +
                           (c1 * (TXZ[p] - TXZ[p - 1]) + c2 * (TXZ[p - 2] - TXZ[p + 1])) * idz;
          const float az = (c1 * (TXZ[p + S] - TXZ[p]) + c2 * (TXZ[p - S] - TXZ[p + 2 * S])) * idx +
                           (c1 * (TZZ[p + 1] - TZZ[p]) + c2 * (TZZ[p - 1] - TZZ[p + 2])) * idz;
          const int cnt = min(min(gz + 1, nz - gz), min(gx + 1, nx - gx));
          const float tp = cnt < np ? TAP[cnt] : 1.0f;
          const float bdt = b * dtv;
          vx = tp * (vx + bdt * ax);
          vz = tp * (vz + bdt * az);
        }
        if (x_box && gz >= pl.z0 && gz < pl.z0 + pl.h)
          tma::inject(d, it, gx * nz + gz, gx, gz, b, vx, vz);
        VX[p] = vx;
        VZ[p] = vz;
        if (ru >= 0) {
          up[0][ru + gz] = vx;
          up[1][ru + gz] = vz;
        }
        if (rd >= 0) {
          dn[0][rd + gz] = vx;
          dn[1][rd + gz] = vz;
        }
      }
    }
    cl.sync();
  }

  // Final state of the own rows.
  const fast::Fields out = d.set[parity ^ (n_steps & 1)];
  float *dst[5] = {out.vx, out.vz, out.txx, out.tzz, out.txz};
  for (int lr = 2 + warp; lr < rows + 2; lr += WARPS) {
    const size_t row = (size_t)(x0 - 2 + lr) * ps;
    for (int z = lane; z < nz; z += 32)
      for (int f = 0; f < 5; ++f) dst[f][row + z] = F[f][lr * S + z];
  }
}

template <bool ADJ>
__global__ void __launch_bounds__(NT, 1)
    cluster_steps(const __grid_constant__ tma::SimDesc d, int nc, int it0, int n_steps,
                  int parity, int store) {
  member_steps<ADJ>(d, nc, it0, n_steps, parity, store);
}

// Forward steps 0 .. n_steps - 1 of a batch: cluster m (CTAs m nc ..
// m nc + nc - 1) runs simulation sims[m] from set 0; a cluster whose flag in
// `active` is zero returns at once (the whole cluster: no barrier is left
// waiting). Two CTAs per SM, so that twice as many clusters run at once.
__global__ void __launch_bounds__(NT, 2)
    cluster_steps_batch(const tma::SimDesc *__restrict__ sims, const int *__restrict__ active,
                        int nc, int n_steps, int store) {
  const int m = (int)(blockIdx.x / (unsigned)nc);
  if (active && !active[m]) return;
  member_steps<false>(sims[m], nc, 0, n_steps, 0, store);
}

template <bool ADJ>
bool configure(size_t smem, int nc) {
  if (cudaFuncSetAttribute(cluster_steps<ADJ>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           (int)smem) != cudaSuccess)
    return false;
  if (nc > 8 &&
      cudaFuncSetAttribute(cluster_steps<ADJ>, cudaFuncAttributeNonPortableClusterSizeAllowed,
                           1) != cudaSuccess)
    return false;
  return true;
}

template <bool ADJ>
bool placeable(size_t smem, int nc) {
  cudaLaunchConfig_t lc = {};
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = nc;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  lc.gridDim = dim3(nc);
  lc.blockDim = dim3(NT);
  lc.dynamicSmemBytes = smem;
  lc.attrs = attr;
  lc.numAttrs = 1;
  int n = 0;
  return cudaOccupancyMaxActiveClusters(&n, cluster_steps<ADJ>, &lc) == cudaSuccess && n >= 1;
}

bool configure_batch(size_t smem, int nc) {
  if (cudaFuncSetAttribute(cluster_steps_batch, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           (int)smem) != cudaSuccess)
    return false;
  if (nc > 8 &&
      cudaFuncSetAttribute(cluster_steps_batch, cudaFuncAttributeNonPortableClusterSizeAllowed,
                           1) != cudaSuccess)
    return false;
  return true;
}

bool placeable_batch(size_t smem, int nc) {
  cudaLaunchConfig_t lc = {};
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = nc;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  lc.gridDim = dim3(nc);
  lc.blockDim = dim3(NT);
  lc.dynamicSmemBytes = smem;
  lc.attrs = attr;
  lc.numAttrs = 1;
  int n = 0;
  return cudaOccupancyMaxActiveClusters(&n, cluster_steps_batch, &lc) == cudaSuccess && n >= 1;
}

}  // namespace

int plan_batch(const int *nx, const int *nz, const int *np, int n, size_t *smem_out) {
  int dev = 0, optin = 0;
  if (n <= 0 || cudaGetDevice(&dev) != cudaSuccess ||
      cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) !=
          cudaSuccess)
    return 0;
  for (int nc : {16, 8}) {
    size_t smem = 0;
    bool fits = true;
    for (int k = 0; k < n && fits; ++k) {
      if (nx[k] < 2 * nc) fits = false;
      smem = std::max(smem, smem_bytes(max_rows(nc, nx[k]), stride(nz[k]), np[k]));
    }
    if (!fits || smem > (size_t)optin) continue;
    if (!configure_batch((size_t)optin, nc)) continue;
    if (placeable_batch(smem, nc)) {
      if (smem_out) *smem_out = smem;
      return nc;
    }
  }
  cudaGetLastError();  // a refused non-portable size is not an error here
  return 0;
}

cudaError_t steps_batch(const tma::SimDesc *sims, const int *active, int n, int nc, size_t smem,
                        int n_steps, bool store, cudaStream_t s) {
  if (n_steps <= 0 || n <= 0) return cudaSuccess;
  cudaLaunchConfig_t lc = {};
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = nc;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  lc.gridDim = dim3((unsigned)(n * nc));
  lc.blockDim = dim3(NT);
  lc.dynamicSmemBytes = smem;
  lc.stream = s;
  lc.attrs = attr;
  lc.numAttrs = 1;
  return cudaLaunchKernelEx(&lc, cluster_steps_batch, sims, active, nc, n_steps, store ? 1 : 0);
}

int plan(int nx, int nz, int np) {
  int dev = 0, optin = 0;
  if (cudaGetDevice(&dev) != cudaSuccess ||
      cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) !=
          cudaSuccess)
    return 0;
  // The shared-memory limit is an attribute of the kernel, shared by every
  // model: set it to the device's maximum, not to this grid's need.
  for (int nc : {16, 8}) {
    if (nx < 2 * nc) continue;
    const size_t smem = smem_bytes(max_rows(nc, nx), stride(nz), np);
    if (smem > (size_t)optin) continue;
    if (!configure<false>((size_t)optin, nc) || !configure<true>((size_t)optin, nc)) continue;
    if (placeable<false>(smem, nc) && placeable<true>(smem, nc)) return nc;
  }
  cudaGetLastError();  // a refused non-portable size is not an error here
  return 0;
}

cudaError_t steps(const tma::SimDesc &d, bool adjoint, int it0, int n_steps, int parity,
                  bool store, int nc, cudaStream_t s) {
  if (n_steps <= 0) return cudaSuccess;
  const size_t smem = smem_bytes(max_rows(nc, d.nx), stride(d.nz), d.np);
  cudaLaunchConfig_t lc = {};
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = nc;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  lc.gridDim = dim3(nc);
  lc.blockDim = dim3(NT);
  lc.dynamicSmemBytes = smem;
  lc.stream = s;
  lc.attrs = attr;
  lc.numAttrs = 1;
  const int st = store ? 1 : 0;
  return adjoint ? cudaLaunchKernelEx(&lc, cluster_steps<true>, d, nc, it0, n_steps, parity, st)
                 : cudaLaunchKernelEx(&lc, cluster_steps<false>, d, nc, it0, n_steps, parity, st);
}

}  // namespace cluster
}  // namespace psv
