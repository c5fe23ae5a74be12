// FP32 production time step: one fused kernel per step.
//
// Each CTA owns a TX x TZ tile of output points. It stages the old
// velocities over the tile plus a 4-point halo in shared memory, computes the
// new stresses over the tile plus a 2-point halo (the halo points are
// recomputed by the neighbouring CTAs too), keeps them in shared memory, and
// finishes with the new velocities of its own points. Old and new wave
// fields live in separate buffers (ping-pong), so neighbouring CTAs never
// see half-updated values and one launch covers the whole step.
//
// Per point and step this moves 16 words instead of the 21 of two separate
// half-step launches, and halves the launches. The arithmetic is the
// reference's stencil (src/fdModel.cpp:599-678 forward, 864-948 adjoint)
// in float with reciprocal multiplies; snapshot storage
// (src/fdModel.cpp:555-572), kernel correlation (src/fdModel.cpp:817-861,
// FP64 accumulation), receiver sampling (src/fdModel.cpp:576-596) and
// source / adjoint-source injection (src/fdModel.cpp:681-751, 951-958) are
// fused in.
#include <cuda_runtime.h>

#include <cstdint>

#include "psv_fast.hpp"

namespace psv {
namespace fast {
namespace {

constexpr int TX = 32, TZ = 64, NT = 256;
constexpr int VXD = TX + 8, VZD = TZ + 8;  // old-velocity tile with 4-point halo
constexpr int SXD = TX + 4, SZD = TZ + 4;  // new-stress tile with 2-point halo
constexpr int kSmemBytes = (2 * VXD * VZD + 3 * SXD * SZD) * 4;

__device__ __forceinline__ float taper(const StepArgs &a, int gx, int gz) {
  // Points at least np frames deep have taper exp(0) = 1 exactly.
  int c = min(min(gx + 1, gz + 1), min(a.nx - gx, a.nz - gz));
  return c < a.np ? __ldg(a.taper_tab + c) : 1.0f;
}

__device__ __forceinline__ void correlate(const StepArgs &a, size_t g, size_t gp, float vx,
                                          float vz, float txx, float tzz, float txz) {
  const float lm = a.lm[gp], la = a.la[gp], mu = a.mu[gp];
  const float avx = a.asnap[0][g], avz = a.asnap[1][g], atxx = a.asnap[2][g],
              atzz = a.asnap[3][g], atxz = a.asnap[4][g];
  const float r = la / lm;
  const float d = lm - la * r;
  const float inv_den = 1.0f / (d * d);
  const float fxx = txx - tzz * r, fzz = tzz - txx * r;
  const float axx = atxx - atzz * r, azz = atzz - atxx * r;
  const float lam = (axx + azz) * (fxx + fzz) * inv_den;
  const float muk = (fxx * axx + fzz * azz) * inv_den + 2.0f * (txz * atxz / (4.0f * mu * mu));
  a.krho[g] -= a.sidt * static_cast<double>(avx * vx + avz * vz);
  a.klam[g] += a.sidt * static_cast<double>(lam);
  a.kmu[g] += a.sidt * 2.0 * static_cast<double>(muk);
}

__device__ __forceinline__ void inject(const StepArgs &a, size_t g, int gx, int gz, float b,
                                       float &vx, float &vz) {
  const InjPlan &p = a.plan;
  int k = p.map[(gx - p.x0) * p.h + (gz - p.z0)];
  if (k < 0) return;
  for (; k < p.n && p.terms[k].cell == (int)g; ++k) {
    const InjTerm t = p.terms[k];
    double term;
    if (t.kind == 0) {
      term = (((t.coef * a.stf[(size_t)t.index * a.nt + a.it]) * a.dt_d) * (double)b) / t.div;
    } else {
      const double *src = t.field == 0 ? a.a_ux : a.a_uz;
      term = ((a.dt_d * (double)b) * src[(size_t)t.index * a.nt + a.it]) / t.div;
    }
    if (t.field == 0)
      vx += (float)term;
    else
      vz += (float)term;
  }
}

template <bool ADJ>
__global__ void __launch_bounds__(NT, 4) fused_step(const StepArgs a) {
  extern __shared__ float smem[];
  float(*sv)[VXD][VZD] = reinterpret_cast<float(*)[VXD][VZD]>(smem);
  float(*st)[SXD][SZD] = reinterpret_cast<float(*)[SXD][SZD]>(smem + 2 * VXD * VZD);
  const int nx = a.nx, nz = a.nz, ps = a.pitch;
  const int X0 = blockIdx.y * TX, Z0 = blockIdx.x * TZ;
  const float c1 = 9.0f / 8.0f, c2 = 1.0f / 24.0f;

  // Receivers read the pre-step velocities (nothing writes the input buffer).
  if (!ADJ && a.rec_vx && blockIdx.x == 0 && blockIdx.y == 0) {
    for (int r = threadIdx.x; r < a.nr; r += NT) {
      const int c = a.rec_cell[r];
      a.rec_vx[(size_t)r * a.nt + a.it] = a.in.vx[c];
      a.rec_vz[(size_t)r * a.nt + a.it] = a.in.vz[c];
    }
  }

  // Phase A: old velocities over the tile + 4-point halo (zero outside).
  // All of a thread's loads are issued before any is stored, so they are in
  // flight together.
  {
    constexpr int N = VXD * VZD, K = (N + NT - 1) / NT;
    float rx[K], rz[K];
#pragma unroll
    for (int k = 0; k < K; ++k) {
      const int e = threadIdx.x + k * NT;
      const int lx = e / VZD, lz = e - lx * VZD;
      const int gx = X0 - 4 + lx, gz = Z0 - 4 + lz;
      rx[k] = 0.f;
      rz[k] = 0.f;
      if (e < N && gx >= 0 && gx < nx && gz >= 0 && gz < nz) {
        const size_t g = (size_t)gx * ps + gz;
        rx[k] = __ldg(a.in.vx + g);
        rz[k] = __ldg(a.in.vz + g);
      }
    }
#pragma unroll
    for (int k = 0; k < K; ++k) {
      const int e = threadIdx.x + k * NT;
      if (e < N) {
        const int lx = e / VZD, lz = e - lx * VZD;
        sv[0][lx][lz] = rx[k];
        sv[1][lx][lz] = rz[k];
      }
    }
  }
  __syncthreads();

  // Phase B: new stresses over the tile + 2-point halo, in chunks of CH
  // points per thread whose loads are issued together.
  {
    constexpr int N = SXD * SZD, K = (N + NT - 1) / NT, CH = ADJ ? 3 : 5;
    const float(*VX)[VZD] = sv[0];
    const float(*VZ)[VZD] = sv[1];
#pragma unroll
    for (int k0 = 0; k0 < K; k0 += CH) {
      float txx[CH], tzz[CH], txz[CH], lm[CH], la[CH], mu[CH];
#pragma unroll
      for (int j = 0; j < CH; ++j) {
        const int e = threadIdx.x + (k0 + j) * NT;
        const int lx = e / SZD, lz = e - lx * SZD;
        const int gx = X0 - 2 + lx, gz = Z0 - 2 + lz;
        txx[j] = tzz[j] = txz[j] = 0.f;
        lm[j] = la[j] = mu[j] = 0.f;
        if (k0 + j < K && e < N && gx >= 0 && gx < nx && gz >= 0 && gz < nz) {
          const size_t g = (size_t)gx * ps + gz;
          txx[j] = __ldg(a.in.txx + g);
          tzz[j] = __ldg(a.in.tzz + g);
          txz[j] = __ldg(a.in.txz + g);
          lm[j] = __ldg(a.lm + g);
          la[j] = __ldg(a.la + g);
          mu[j] = __ldg(a.mu + g);
        }
      }
#pragma unroll
      for (int j = 0; j < CH; ++j) {
        const int e = threadIdx.x + (k0 + j) * NT;
        if (k0 + j >= K || e >= N) continue;
        const int lx = e / SZD, lz = e - lx * SZD;
        const int gx = X0 - 2 + lx, gz = Z0 - 2 + lz;
        float sxx = txx[j], szz = tzz[j], sxz = txz[j];
        if (gx >= 0 && gx < nx && gz >= 0 && gz < nz) {
          const size_t g = (size_t)gx * nz + gz;   // unpadded (snapshots, kernels)
          const size_t gp = (size_t)gx * ps + gz;  // padded (wave fields, medium)
          const bool own = lx >= 2 && lx < TX + 2 && lz >= 2 && lz < TZ + 2;
          const int vx_ = lx + 2, vz_ = lz + 2;  // this point in the velocity tile
          if (own && a.snap[0]) {
            a.snap[0][g] = VX[vx_][vz_];
            a.snap[1][g] = VZ[vx_][vz_];
            a.snap[2][g] = sxx;
            a.snap[3][g] = szz;
            a.snap[4][g] = sxz;
          }
          if (ADJ && own && a.asnap[0] && gx >= a.fx0 && gx < a.fx1 && gz >= a.fz0 &&
              gz < a.fz1)
            correlate(a, g, gp, VX[vx_][vz_], VZ[vx_][vz_], sxx, szz, sxz);
          if (gx >= 2 && gx < nx - 2 && gz >= 2 && gz < nz - 2) {
            const float dvx = c1 * (VX[vx_ + 1][vz_] - VX[vx_][vz_]) +
                              c2 * (VX[vx_ - 1][vz_] - VX[vx_ + 2][vz_]);
            const float dvz = c1 * (VZ[vx_][vz_] - VZ[vx_][vz_ - 1]) +
                              c2 * (VZ[vx_][vz_ - 2] - VZ[vx_][vz_ + 1]);
            const float gxz = (c1 * (VX[vx_][vz_ + 1] - VX[vx_][vz_]) +
                               c2 * (VX[vx_][vz_ - 1] - VX[vx_][vz_ + 2])) * a.idz +
                              (c1 * (VZ[vx_][vz_] - VZ[vx_ - 1][vz_]) +
                               c2 * (VZ[vx_ - 2][vz_] - VZ[vx_ + 1][vz_])) * a.idx;
            const float ex = dvx * a.idx, ez = dvz * a.idz;
            const float tp = taper(a, gx, gz);
            const float dt = ADJ ? -a.dt : a.dt;
            sxx = tp * (sxx + dt * (lm[j] * ex + la[j] * ez));
            szz = tp * (szz + dt * (la[j] * ex + lm[j] * ez));
            sxz = tp * (sxz + dt * mu[j] * gxz);
          }
          if (own) {
            a.out.txx[gp] = sxx;
            a.out.tzz[gp] = szz;
            a.out.txz[gp] = sxz;
          }
        }
        st[0][lx][lz] = sxx;
        st[1][lx][lz] = szz;
        st[2][lx][lz] = sxz;
      }
    }
  }
  __syncthreads();

  // Phase C: new velocities of the tile's own points.
  {
    constexpr int K = TX * TZ / NT;
    const float(*TXX)[SZD] = st[0];
    const float(*TZZ)[SZD] = st[1];
    const float(*TXZ)[SZD] = st[2];
    const InjPlan &p = a.plan;
    float bb[K];
#pragma unroll
    for (int k = 0; k < K; ++k) {
      const int e = threadIdx.x + k * NT;
      const int gx = X0 + e / TZ, gz = Z0 + e % TZ;
      bb[k] = (gx < nx && gz < nz) ? __ldg(a.b + (size_t)gx * ps + gz) : 0.f;
    }
#pragma unroll
    for (int k = 0; k < K; ++k) {
      const int e = threadIdx.x + k * NT;
      const int lx = e / TZ, lz = e % TZ;
      const int gx = X0 + lx, gz = Z0 + lz;
      if (gx >= nx || gz >= nz) continue;
      const size_t g = (size_t)gx * nz + gz;   // unpadded (injection cells)
      const size_t gp = (size_t)gx * ps + gz;  // padded
      float vx = sv[0][lx + 4][lz + 4], vz = sv[1][lx + 4][lz + 4];
      const float b = bb[k];
      if (gx >= 2 && gx < nx - 2 && gz >= 2 && gz < nz - 2) {
        const int sx = lx + 2, sz = lz + 2;
        const float ax = (c1 * (TXX[sx][sz] - TXX[sx - 1][sz]) +
                          c2 * (TXX[sx - 2][sz] - TXX[sx + 1][sz])) * a.idx +
                         (c1 * (TXZ[sx][sz] - TXZ[sx][sz - 1]) +
                          c2 * (TXZ[sx][sz - 2] - TXZ[sx][sz + 1])) * a.idz;
        const float az = (c1 * (TXZ[sx + 1][sz] - TXZ[sx][sz]) +
                          c2 * (TXZ[sx - 1][sz] - TXZ[sx + 2][sz])) * a.idx +
                         (c1 * (TZZ[sx][sz + 1] - TZZ[sx][sz]) +
                          c2 * (TZZ[sx][sz - 1] - TZZ[sx][sz + 2])) * a.idz;
        const float tp = taper(a, gx, gz);
        const float bdt = b * (ADJ ? -a.dt : a.dt);
        vx = tp * (vx + bdt * ax);
        vz = tp * (vz + bdt * az);
      }
      if (p.n && gx >= p.x0 && gx < p.x0 + p.w && gz >= p.z0 && gz < p.z0 + p.h)
        inject(a, g, gx, gz, b, vx, vz);
      a.out.vx[gp] = vx;
      a.out.vz[gp] = vz;
    }
  }
}

template <bool ADJ>
cudaError_t launch(const StepArgs &a, cudaStream_t s) {
  // The shared-memory opt-in is a per-device attribute: set it once per device.
  static unsigned long long configured = 0;
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  const unsigned long long bit = 1ull << (dev & 63);
  if (!(configured & bit)) {
    e = cudaFuncSetAttribute(fused_step<ADJ>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             kSmemBytes);
    if (e != cudaSuccess) return e;
    configured |= bit;
  }
  const dim3 grid((a.nz + TZ - 1) / TZ, (a.nx + TX - 1) / TX);
  fused_step<ADJ><<<grid, NT, kSmemBytes, s>>>(a);
  return cudaGetLastError();
}

cudaError_t zero(const SolverArgs &a, void *const second[5], cudaStream_t s) {
  const size_t bytes = (size_t)a.nx * a.pitch * sizeof(float);
  void *prim[5] = {a.vx, a.vz, a.txx, a.tzz, a.txz};
  for (int f = 0; f < 5; ++f) {
    cudaError_t e = cudaMemsetAsync(prim[f], 0, bytes, s);
    if (e == cudaSuccess) e = cudaMemsetAsync(second[f], 0, bytes, s);
    if (e != cudaSuccess) return e;
  }
  return cudaSuccess;
}

}  // namespace

StepArgs base_step_args(const SolverArgs &a) {
  StepArgs s;
  s.nx = a.nx;
  s.nz = a.nz;
  s.pitch = a.pitch;
  s.np = a.np;
  s.nt = a.nt;
  s.dt = (float)a.dt;
  s.dt_d = a.dt;
  s.idx = (float)(1.0 / a.dx);
  s.idz = (float)(1.0 / a.dz);
  s.lm = (const float *)a.lm;
  s.la = (const float *)a.la;
  s.mu = (const float *)a.mu;
  s.b = (const float *)a.b;
  s.taper_tab = (const float *)a.taper_tab;
  return s;
}

void set_step_buffers(StepArgs &s, const SolverArgs &a, void *const second[5], int cur) {
  void *prim[5] = {a.vx, a.vz, a.txx, a.tzz, a.txz};
  void *const *src = cur == 0 ? prim : second;
  void *const *dst = cur == 0 ? second : prim;
  s.in = ConstFields{(const float *)src[0], (const float *)src[1], (const float *)src[2],
                     (const float *)src[3], (const float *)src[4]};
  s.out = Fields{(float *)dst[0], (float *)dst[1], (float *)dst[2], (float *)dst[3],
                 (float *)dst[4]};
}

cudaError_t step(const StepArgs &a, bool adjoint, cudaStream_t s) {
  return adjoint ? launch<true>(a, s) : launch<false>(a, s);
}

cudaError_t forward(const SolverArgs &a, void *const second[5], int *cur, const InjPlan &plan,
                    int shot, bool store, int it0, int it1, bool zero_first, bool finish,
                    cudaStream_t s) {
  if (zero_first) {
    cudaError_t e = zero(a, second, s);
    if (e != cudaSuccess) return e;
    *cur = 0;
  }
  StepArgs sa = base_step_args(a);
  sa.plan = plan;
  sa.stf = a.stf;
  sa.rec_cell = a.rec_cell;
  sa.nr = a.nr;
  float *raw = (float *)a.rec_raw;
  sa.rec_vx = a.nr ? raw : nullptr;
  sa.rec_vz = a.nr ? raw + (size_t)a.nr * a.nt : nullptr;
  const size_t gsz = (size_t)a.nx * a.nz;
  for (int it = it0; it < it1; ++it) {
    sa.it = it;
    for (int f = 0; f < 5; ++f)
      sa.snap[f] = (store && it % a.si == 0)
                       ? (float *)a.accu[f] + ((size_t)shot * a.snapshots + it / a.si) * gsz
                       : nullptr;
    set_step_buffers(sa, a, second, *cur);
    cudaEvent_t *ev = a.events ? a.events + 2 * (it - it0) : nullptr;
    if (ev) cudaEventRecord(ev[0], s);
    cudaError_t e = launch<false>(sa, s);
    if (ev) cudaEventRecord(ev[1], s);
    if (e != cudaSuccess) return e;
    *cur ^= 1;
  }
  if (finish && a.nr) {
    const size_t off = (size_t)shot * a.nr * a.nt;
    receiver_cumsum_f32(a.nr, a.nt, it1, a.dt, a.dx * a.dz, sa.rec_vx, sa.rec_vz,
                        a.rtf_ux + off, a.rtf_uz + off, s);
  }
  return cudaGetLastError();
}

cudaError_t adjoint(const SolverArgs &a, void *const second[5], int *cur, const InjPlan &plan,
                    int shot, cudaStream_t s) {
  cudaError_t e = zero(a, second, s);
  if (e != cudaSuccess) return e;
  *cur = 0;
  StepArgs sa = base_step_args(a);
  sa.plan = plan;
  sa.a_ux = a.a_stf_ux + (size_t)shot * a.nr * a.nt;
  sa.a_uz = a.a_stf_uz + (size_t)shot * a.nr * a.nt;
  sa.krho = a.k_rho;
  sa.klam = a.k_lam;
  sa.kmu = a.k_mu;
  sa.sidt = a.si * a.dt;
  sa.fx0 = a.fx0;
  sa.fx1 = a.fx1;
  sa.fz0 = a.fz0;
  sa.fz1 = a.fz1;
  const size_t gsz = (size_t)a.nx * a.nz;
  for (int it = a.nt - 1; it >= 0; --it) {
    sa.it = it;
    for (int f = 0; f < 5; ++f)
      sa.asnap[f] = (it % a.si == 0)
                        ? (const float *)a.accu[f] + ((size_t)shot * a.snapshots + it / a.si) * gsz
                        : nullptr;
    set_step_buffers(sa, a, second, *cur);
    e = launch<true>(sa, s);
    if (e != cudaSuccess) return e;
    *cur ^= 1;
  }
  return cudaGetLastError();
}

}  // namespace fast
}  // namespace psv
