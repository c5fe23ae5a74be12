// FP32 exact adjoint step with TMA tile loads.
//
// The transpose of the forward step (notation and algebra in psv_exact.cuh):
// per step n, from l^{n+1} = (lv, lt), the forward states v^n and tau^{n+1}
// and the medium, it produces l^n = (v-bar, tau-bar) and adds the step's
// terms to the gradients of lm, la, mu and b. Each CTA owns a
// kTX x kTZ tile. Thread 0 issues fourteen tiled bulk-tensor copies that
// complete on one mbarrier: b, lv with a 4-point halo in both axes; lt, lm,
// mu, v^n and tau^{n+1} with a 2-point halo (lambda = lm - 2 mu, formed in
// registers as the forward TMA step forms it) (all boxes kTZ + 8 wide,
// starting 4 columns left of the tile so that they stay 16-byte aligned;
// the copies zero-fill outside the grid). The medium is issued before the
// programmatic-dependent-launch wait (it does not change during a gradient),
// the rest after it. Then, in shared memory:
//   phase 1: w = b dt T lv over the tile + 4;
//   phase 2: lt~ = lt + A^T w (in place) and p = dt C y over the tile + 2
//            (in place of lm, la, mu: each point reads only its own);
//   phase 3: per own point, tau-bar = T lt~, v-bar = T lv + E^T p plus the
//            receiver terms of the point (in increasing receiver index), and
//            the gradient terms, added to sums loaded right after the wait.
// The adjoint state is computed with the expressions of
// exact::exact_step_tile<float> and exact::add_receiver_terms: the general
// path gives the same bits; the interior path below drops the taper factor
// (exactly 1), so the compiler fuses a few products differently there
// (about 4e-7 relative on a gradient). The gradient terms are formed in
// FP32 and summed in float-float
// pairs (hi, lo) with Knuth's TwoSum (The Art of Computer Programming,
// vol. 2, 4.2.2), which carries each addition's rounding error exactly into
// lo: about 48 significant bits, like the FP64 sums of exact_step_tile, but
// on the FP32 pipes (GB300 issues FP64 at a small fraction of the FP32
// rate, and FP64 sums were most of this kernel's time). finish() turns the
// pairs into FP64 once per gradient. With Step::g_part set, each step's
// terms first go into an FP32 partial sum per point (one float4 for lm, la,
// mu, b), which the flush steps (every few steps, and the last) add into
// the pairs: per step the kernel then reads and writes 16 bytes of sums per
// point instead of 32 (the pairs' traffic on flush steps only).
//
// Tiles whose 4-halo region lies inside the updated region and at least np
// frames deep (taper exactly 1) and that hold no source point take a path
// without per-point tests.
//
// The mbarrier wait is bounded: on time-out the CTA raises the error flag,
// waits (bounded again) for its copies to land, and returns.
#include "psv_exact_tma.hpp"

#include <algorithm>
#include <cstdint>

#include "psv_tma.hpp"
#include "psv_tma_ptx.cuh"

namespace psv {
namespace exact_tma {
namespace {

using tma::griddep_launch_dependents;
using tma::griddep_wait;
using tma::mbar_wait;
using tma::smem_u32;
using tma::tma_load_2d;
using tma::tma_load_3d;

constexpr int TX = kTX, TZ = kTZ, NT = 256, W = TZ + 8;
constexpr int VR = TX + 8;  // rows of the 4-halo boxes: X0-4 .. X0+TX+4
constexpr int SR = TX + 4;  // rows of the 2-halo boxes: X0-2 .. X0+TX+2
constexpr int PC = TZ + 4;  // columns of phase 2: box columns 2 .. TZ+6
constexpr int VB = VR * W, SB = SR * W;  // floats per box
// Shared layout (floats): copies first, each box a multiple of 128 bytes.
constexpr int OFF_LV = 0;                   // lvx, lvz
constexpr int OFF_B = 2 * VB;               // b
constexpr int OFF_LT = 3 * VB;              // ltxx, ltzz, ltxz (then lt~)
constexpr int OFF_M = OFF_LT + 3 * SB;      // lm, la, mu
constexpr int OFF_FV = OFF_M + 3 * SB;      // vx, vz of v^n
constexpr int OFF_FT = OFF_FV + 2 * SB;     // txx, tzz, txz of tau^{n+1}
constexpr int OFF_W = OFF_FT + 3 * SB;      // wx, wz
constexpr int OFF_P = OFF_M;                // px, pz, q over lm, la, mu (same points)
constexpr int TOTAL = OFF_W + 2 * VB;
// Delivered by the copies: every box but la's (lambda is lm - 2 mu, formed
// in registers as the forward TMA step forms it; its box is left empty and
// later holds p_z).
constexpr int TX_BYTES = (OFF_W - SB) * 4;
constexpr int SMEM = TOTAL * 4 + 16 + 128;  // + mbarrier + alignment slack
constexpr int ROWS = TX / (NT / 32);        // own rows per thread
static_assert((VB * 4) % 128 == 0 && (SB * 4) % 128 == 0, "boxes must stay 128-byte aligned");
static_assert(TZ == 32 && TX % (NT / 32) == 0, "one warp per tile row");

__device__ __forceinline__ float taper_at(const Step &a, int ix, int iz) {
  int c = min(min(ix + 1, iz + 1), min(a.nx - ix, a.nz - iz));
  return a.taper_tab[min(c, a.np)];
}

__device__ __forceinline__ bool interior(const Step &a, int ix, int iz) {
  return ix >= 2 && ix < a.nx - 2 && iz >= 2 && iz < a.nz - 2;
}

// (hi, lo) + x: s = hi + x rounded, and e with s + e == hi + x exactly
// (TwoSum); e goes into lo.
__device__ __forceinline__ float2 ff_add(float2 a, float x) {
  const float s = a.x + x;
  const float bp = s - a.x;
  const float e = (a.x - (s - bp)) + (x - bp);
  return make_float2(s, a.y + e);
}

// Phases 1-3 of one tile (the copies have landed). INNER: every point of
// the 4-halo region is interior with taper 1 and no own point has a source
// term.
template <bool INNER>
__device__ __forceinline__ void tile_body(const Step &a, float *sm, int X0, int Z0,
                                          const float2 *glm, const float2 *gla,
                                          const float2 *gmu, const float2 *gb,
                                          const float4 *gpart) {
  const int tid = threadIdx.x, lane = tid & 31, wr = tid >> 5;
  const int iz = Z0 + lane;
  const float c1 = 9.0f / 8.0f, c2 = 1.0f / 24.0f;
  const float *LVX = sm + OFF_LV, *LVZ = sm + OFF_LV + VB, *B = sm + OFF_B;
  float *WX = sm + OFF_W, *WZ = sm + OFF_W + VB;
  // Phase 1: w = b dt T lv at interior points, 0 elsewhere.
  for (int k = tid; k < VB; k += NT) {
    const int r = k / W, c = k - r * W;
    const int ix = X0 - 4 + r, jz = Z0 - 4 + c;
    float wx = 0.f, wz = 0.f;
    if (INNER) {
      const float s = B[k] * a.dt;
      wx = s * LVX[k];
      wz = s * LVZ[k];
    } else if (ix >= 0 && ix < a.nx && jz >= 0 && jz < a.nz && interior(a, ix, jz)) {
      const float s = B[k] * a.dt * taper_at(a, ix, jz);
      wx = s * LVX[k];
      wz = s * LVZ[k];
    }
    WX[k] = wx;
    WZ[k] = wz;
  }
  __syncthreads();

  float *LXX = sm + OFF_LT, *LZZ = sm + OFF_LT + SB, *LXZ = sm + OFF_LT + 2 * SB;
  const float *LM = sm + OFF_M, *MU = sm + OFF_M + 2 * SB;
  float *PX = sm + OFF_P, *PZ = sm + OFF_P + SB, *QQ = sm + OFF_P + 2 * SB;
  // Phase 2: lt~ = lt - (A^T w terms), and p_x = dt (lm y_xx + la y_zz),
  // p_z = dt (la y_xx + lm y_zz), q = dt mu y_xz with y = T lt~ on I, 0
  // elsewhere; over rows X0-2 .. X0+TX+1 and columns Z0-2 .. Z0+TZ+1.
  for (int k = tid; k < SR * PC; k += NT) {
    const int r = k / PC, c = 2 + (k - r * PC);
    const int ix = X0 - 2 + r, jz = Z0 - 4 + c;
    const int s = r * W + c;        // in the 2-halo boxes
    const int v = (r + 2) * W + c;  // the same point in the 4-halo boxes
    float px = 0.f, pz = 0.f, q = 0.f;
    if (INNER || (ix >= 0 && ix < a.nx && jz >= 0 && jz < a.nz)) {
      const float dxp_wx = c1 * (WX[v + W] - WX[v]) + c2 * (WX[v - W] - WX[v + 2 * W]);
      const float dzp_wx = c1 * (WX[v + 1] - WX[v]) + c2 * (WX[v - 1] - WX[v + 2]);
      const float dzm_wz = c1 * (WZ[v] - WZ[v - 1]) + c2 * (WZ[v - 2] - WZ[v + 1]);
      const float dxm_wz = c1 * (WZ[v] - WZ[v - W]) + c2 * (WZ[v - 2 * W] - WZ[v + W]);
      const float lxx = LXX[s] - dxp_wx * a.idx;
      const float lzz = LZZ[s] - dzm_wz * a.idz;
      const float lxz = LXZ[s] - dzp_wx * a.idz - dxm_wz * a.idx;
      LXX[s] = lxx;
      LZZ[s] = lzz;
      LXZ[s] = lxz;
      if (INNER) {
        const float lm = LM[s], mu = MU[s];
        const float la = lm - 2.0f * mu;
        px = a.dt * (lm * lxx + la * lzz);
        pz = a.dt * (la * lxx + lm * lzz);
        q = a.dt * mu * lxz;
      } else if (interior(a, ix, jz)) {
        const float tp = taper_at(a, ix, jz);
        const float yxx = tp * lxx, yzz = tp * lzz, yxz = tp * lxz;
        if (!(yxx == 0.f && yzz == 0.f && yxz == 0.f)) {
          const float lm = LM[s], mu = MU[s];
          const float la = lm - 2.0f * mu;
          px = a.dt * (lm * yxx + la * yzz);
          pz = a.dt * (la * yxx + lm * yzz);
          q = a.dt * mu * yxz;
        }
      }
    }
    PX[s] = px;
    PZ[s] = pz;
    QQ[s] = q;
  }
  __syncthreads();

  // Phase 3: own points.
  if (!INNER && iz >= a.nz) return;
  const float *FVX = sm + OFF_FV, *FVZ = sm + OFF_FV + SB;
  const float *FXX = sm + OFF_FT, *FZZ = sm + OFF_FT + SB, *FXZ = sm + OFF_FT + 2 * SB;
  const int tile = blockIdx.x;
  const int r0 = a.rec_start[tile], r1 = a.rec_start[tile + 1];
  const int c = lane + 4;
#pragma unroll
  for (int j = 0; j < ROWS; ++j) {
    const int lx = wr + j * (NT / 32);
    const int ix = X0 + lx;
    if (!INNER && ix >= a.nx) break;
    const size_t p = (size_t)ix * a.pitch + iz;
    const size_t u = (size_t)ix * a.nz + iz;
    const int s = (lx + 2) * W + c;  // 2-halo boxes
    const int v = (lx + 4) * W + c;  // 4-halo boxes
    const bool in = INNER || interior(a, ix, iz);
    const float tp = (INNER || !in) ? 1.f : taper_at(a, ix, iz);
    const float lxx = LXX[s], lzz = LZZ[s], lxz = LXZ[s];
    // tau-bar^n
    a.olt[0][p] = tp * lxx;
    a.olt[1][p] = tp * lzz;
    a.olt[2][p] = tp * lxz;
    // E^T (dt C y):  v-bar_x += -D-_x(p_x)/dx - D-_z(q)/dz,
    //                v-bar_z += -D+_z(p_z)/dz - D+_x(q)/dx
    const float dxm_px = c1 * (PX[s] - PX[s - W]) + c2 * (PX[s - 2 * W] - PX[s + W]);
    const float dzm_q = c1 * (QQ[s] - QQ[s - 1]) + c2 * (QQ[s - 2] - QQ[s + 1]);
    const float dzp_pz = c1 * (PZ[s + 1] - PZ[s]) + c2 * (PZ[s - 1] - PZ[s + 2]);
    const float dxp_q = c1 * (QQ[s + W] - QQ[s]) + c2 * (QQ[s - W] - QQ[s + 2 * W]);
    const float lvx = LVX[v], lvz = LVZ[v];
    float ovx = tp * lvx - dxm_px * a.idx - dzm_q * a.idz;
    float ovz = tp * lvz - dzp_pz * a.idz - dxp_q * a.idx;
    // Receiver terms v-bar^n(rec) += adj[r][n].
    for (int i = r0; i < r1; ++i) {
      const int rr = a.rec_list[i];
      if (a.rec_cell[rr] == (int)p) {
        ovx = ovx + (float)a.adj_x[(size_t)rr * a.nt + a.it];
        ovz = ovz + (float)a.adj_z[(size_t)rr * a.nt + a.it];
      }
    }
    a.olv[0][p] = ovx;
    a.olv[1][p] = ovz;
    float2 g_b = gb[j];
    // With partial sums (a.g_part): this step's terms go into the FP32
    // partial of the point (lm, la, mu, b); on a flush step the partial plus
    // the terms go into the float-float pairs and the partial restarts at 0.
    const bool part = a.g_part != nullptr;
    float4 gq = gpart[j];
    float t_lm = 0.f, t_la = 0.f, t_mu = 0.f, t_b = 0.f;
    if (in) {
      // grad_b += dt T lv . A tau^{n+1}
      const float ax = (c1 * (FXX[s] - FXX[s - W]) + c2 * (FXX[s - 2 * W] - FXX[s + W])) * a.idx +
                       (c1 * (FXZ[s] - FXZ[s - 1]) + c2 * (FXZ[s - 2] - FXZ[s + 1])) * a.idz;
      const float az = (c1 * (FXZ[s + W] - FXZ[s]) + c2 * (FXZ[s - W] - FXZ[s + 2 * W])) * a.idx +
                       (c1 * (FZZ[s + 1] - FZZ[s]) + c2 * (FZZ[s - 1] - FZZ[s + 2])) * a.idz;
      t_b = (a.dt * tp) * (lvx * ax + lvz * az);
      if (!part) g_b = ff_add(g_b, t_b);
      // Medium gradients from the strain rates of v^n.
      const float ex = (c1 * (FVX[s + W] - FVX[s]) + c2 * (FVX[s - W] - FVX[s + 2 * W])) * a.idx;
      const float ez = (c1 * (FVZ[s] - FVZ[s - 1]) + c2 * (FVZ[s - 2] - FVZ[s + 1])) * a.idz;
      const float gxz = (c1 * (FVX[s + 1] - FVX[s]) + c2 * (FVX[s - 1] - FVX[s + 2])) * a.idz +
                        (c1 * (FVZ[s] - FVZ[s - W]) + c2 * (FVZ[s - 2 * W] - FVZ[s + W])) * a.idx;
      const float yxx = tp * lxx, yzz = tp * lzz, yxz = tp * lxz;
      t_lm = a.dt * (yxx * ex + yzz * ez);
      t_la = a.dt * (yxx * ez + yzz * ex);
      t_mu = a.dt * yxz * gxz;
      if (!part) {
        a.g_lm[u] = ff_add(glm[j], t_lm);
        a.g_la[u] = ff_add(gla[j], t_la);
        a.g_mu[u] = ff_add(gmu[j], t_mu);
      }
    }
    // Source terms s = coef stf dt b / div at their points depend on b.
    const InjPlan &pl = a.plan;
    bool src = false;
    if (!INNER && pl.n && ix >= pl.x0 && ix < pl.x0 + pl.w && iz >= pl.z0 && iz < pl.z0 + pl.h) {
      int k = pl.map[(ix - pl.x0) * pl.h + (iz - pl.z0)];
      for (; k >= 0 && k < pl.n && pl.terms[k].cell == (int)u; ++k) {
        const InjTerm t = pl.terms[k];
        if (t.kind != 0) continue;
        const double ds = ((t.coef * a.stf[(size_t)t.index * a.nt + a.it]) * a.dt_d) / t.div;
        const float ts = (float)(ds * (double)(t.field == 0 ? lvx : lvz));
        if (part)
          t_b += ts;
        else
          g_b = ff_add(g_b, ts);
        src = true;
      }
    }
    if (!part) {
      if (in || src) a.g_b[u] = g_b;
      continue;
    }
    gq.x += t_lm;
    gq.y += t_la;
    gq.z += t_mu;
    gq.w += t_b;
    if (a.flush) {
      a.g_lm[u] = ff_add(glm[j], gq.x);
      a.g_la[u] = ff_add(gla[j], gq.y);
      a.g_mu[u] = ff_add(gmu[j], gq.z);
      a.g_b[u] = ff_add(g_b, gq.w);
      a.g_part[u] = make_float4(0.f, 0.f, 0.f, 0.f);
    } else if (in || src) {
      a.g_part[u] = gq;
    }
  }
}

__global__ void __launch_bounds__(NT, 4)
    exact_step_tma(const __grid_constant__ Maps maps, const Step a, int tiles_z) {
  extern __shared__ unsigned char smem_raw[];
  float *sm = reinterpret_cast<float *>(
      (reinterpret_cast<uintptr_t>(smem_raw) + 127) & ~static_cast<uintptr_t>(127));
  uint64_t *bar = reinterpret_cast<uint64_t *>(sm + TOTAL);
  const int tx = blockIdx.x / tiles_z, tz = blockIdx.x - tx * tiles_z;
  const int X0 = tx * TX, Z0 = tz * TZ;
  const int tid = threadIdx.x;

  if (tid == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(1)
                 : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)),
                 "r"(TX_BYTES)
                 : "memory");
    tma_load_2d(sm + OFF_B, &maps.b, Z0 - 4, X0 - 4, bar);
    tma_load_2d(sm + OFF_M, &maps.lm, Z0 - 4, X0 - 2, bar);
    tma_load_2d(sm + OFF_M + 2 * SB, &maps.mu, Z0 - 4, X0 - 2, bar);
  }
  __syncthreads();  // the initialised mbarrier, before anyone waits on it
  griddep_wait();
  if (tid == 0) {
    tma_load_3d(sm + OFF_LV, &maps.lam_v, Z0 - 4, X0 - 4, a.lv[0], bar);
    tma_load_3d(sm + OFF_LV + VB, &maps.lam_v, Z0 - 4, X0 - 4, a.lv[1], bar);
    for (int f = 0; f < 3; ++f)
      tma_load_3d(sm + OFF_LT + f * SB, &maps.lam_t, Z0 - 4, X0 - 2, a.lt[f], bar);
    for (int f = 0; f < 2; ++f)
      tma_load_3d(sm + OFF_FV + f * SB, &maps.slots, Z0 - 4, X0 - 2, a.sv + f, bar);
    for (int f = 0; f < 3; ++f)
      tma_load_3d(sm + OFF_FT + f * SB, &maps.slots, Z0 - 4, X0 - 2, a.st + 2 + f, bar);
  }
  griddep_launch_dependents();

  // This thread's own points (column lane, rows w, w + 8, ...) and their
  // gradient sums, loaded while the copies fly.
  const int lane = tid & 31, wr = tid >> 5;
  const int iz = Z0 + lane;
  // (With partial sums, the pairs are read only on flush steps.)
  float2 glm[ROWS], gla[ROWS], gmu[ROWS], gb[ROWS];
  float4 gpart[ROWS];
  const bool pairs = a.g_part == nullptr || a.flush;
#pragma unroll
  for (int j = 0; j < ROWS; ++j) {
    const int ix = X0 + wr + j * (NT / 32);
    glm[j] = gla[j] = gmu[j] = gb[j] = make_float2(0.f, 0.f);
    gpart[j] = make_float4(0.f, 0.f, 0.f, 0.f);
    if (ix < a.nx && iz < a.nz) {
      const size_t u = (size_t)ix * a.nz + iz;
      if (pairs) {
        glm[j] = a.g_lm[u];
        gla[j] = a.g_la[u];
        gmu[j] = a.g_mu[u];
        gb[j] = a.g_b[u];
      }
      if (a.g_part) gpart[j] = a.g_part[u];
    }
  }

  const bool landed = mbar_wait(bar, 0, 1u << 20);
  if (__syncthreads_or(!landed)) {
    if (tid == 0) {
      atomicOr(a.err, 1);
      mbar_wait(bar, 0, 1u << 20);
    }
    return;
  }

  const InjPlan &pl = a.plan;
  const int lo = max(2, a.np - 1);
  const bool inner = X0 - 4 >= lo && Z0 - 4 >= lo &&
                     X0 + TX + 3 <= min(a.nx - 3, a.nx - a.np) &&
                     Z0 + TZ + 3 <= min(a.nz - 3, a.nz - a.np) &&
                     !(pl.n && X0 < pl.x0 + pl.w && pl.x0 < X0 + TX && Z0 < pl.z0 + pl.h &&
                       pl.z0 < Z0 + TZ);
  if (inner)
    tile_body<true>(a, sm, X0, Z0, glm, gla, gmu, gb, gpart);
  else
    tile_body<false>(a, sm, X0, Z0, glm, gla, gmu, gb, gpart);
}

}  // namespace

int tile_count(int nx, int nz) { return ((nx + TX - 1) / TX) * ((nz + TZ - 1) / TZ); }

int tile_of(int nz, int ix, int iz) { return (ix / TX) * ((nz + TZ - 1) / TZ) + iz / TZ; }

bool encode(Maps &m, const float *lam, int n_lam, const float *slots, int n_slot_planes,
            size_t plane_bytes, const float *lm, const float *la, const float *mu, const float *b,
            int nx, int nz, int pitch) {
  return tma::encode_planes(&m.lam_v, lam, n_lam, plane_bytes, nx, nz, pitch, W, VR) &&
         tma::encode_planes(&m.lam_t, lam, n_lam, plane_bytes, nx, nz, pitch, W, SR) &&
         tma::encode_planes(&m.slots, slots, n_slot_planes, plane_bytes, nx, nz, pitch, W, SR) &&
         tma::encode_2d(&m.lm, lm, nx, nz, pitch, W, SR) &&
         tma::encode_2d(&m.la, la, nx, nz, pitch, W, SR) &&
         tma::encode_2d(&m.mu, mu, nx, nz, pitch, W, SR) &&
         tma::encode_2d(&m.b, b, nx, nz, pitch, W, VR);
}

__global__ void ff_finish(size_t n, const float2 *a0, const float2 *a1, const float2 *a2,
                          const float2 *a3, double *o0, double *o1, double *o2, double *o3) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n;
       i += (size_t)gridDim.x * blockDim.x) {
    o0[i] = (double)a0[i].x + (double)a0[i].y;
    o1[i] = (double)a1[i].x + (double)a1[i].y;
    o2[i] = (double)a2[i].x + (double)a2[i].y;
    o3[i] = (double)a3[i].x + (double)a3[i].y;
  }
}

cudaError_t finish(size_t n, float2 *const ff[4], double *const out[4], cudaStream_t s) {
  if (!n) return cudaSuccess;
  const int blocks = (int)std::min<size_t>((n + 255) / 256, 4096);
  ff_finish<<<blocks, 256, 0, s>>>(n, ff[0], ff[1], ff[2], ff[3], out[0], out[1], out[2], out[3]);
  return cudaGetLastError();
}

__global__ void ff_accumulate(size_t n, const float2 *a0, const float2 *a1, const float2 *a2,
                              const float2 *a3, double *o0, double *o1, double *o2, double *o3,
                              int first) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n;
       i += (size_t)gridDim.x * blockDim.x) {
    const double v0 = (double)a0[i].x + (double)a0[i].y, v1 = (double)a1[i].x + (double)a1[i].y;
    const double v2 = (double)a2[i].x + (double)a2[i].y, v3 = (double)a3[i].x + (double)a3[i].y;
    if (first) {
      o0[i] = v0;
      o1[i] = v1;
      o2[i] = v2;
      o3[i] = v3;
    } else {
      o0[i] += v0;
      o1[i] += v1;
      o2[i] += v2;
      o3[i] += v3;
    }
  }
}

cudaError_t accumulate(size_t n, const float2 *const ff[4], double *const out[4], bool first,
                       cudaStream_t s) {
  if (!n) return cudaSuccess;
  const int blocks = (int)std::min<size_t>((n + 255) / 256, 4096);
  ff_accumulate<<<blocks, 256, 0, s>>>(n, ff[0], ff[1], ff[2], ff[3], out[0], out[1], out[2],
                                       out[3], first ? 1 : 0);
  return cudaGetLastError();
}

cudaError_t step(const Maps &maps, const Step &a, cudaStream_t s) {
  static unsigned long long configured = 0;
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  const unsigned long long bit = 1ull << (dev & 63);
  if (!(configured & bit)) {
    e = cudaFuncSetAttribute(exact_step_tma, cudaFuncAttributeMaxDynamicSharedMemorySize, SMEM);
    if (e != cudaSuccess) return e;
    configured |= bit;
  }
  const int tiles_z = (a.nz + TZ - 1) / TZ;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  cudaLaunchConfig_t lc = {};
  lc.gridDim = dim3(tile_count(a.nx, a.nz));
  lc.blockDim = dim3(NT);
  lc.dynamicSmemBytes = SMEM;
  lc.stream = s;
  lc.attrs = attr;
  lc.numAttrs = 1;
  return cudaLaunchKernelEx(&lc, exact_step_tma, maps, a, tiles_z);
}

}  // namespace exact_tma
}  // namespace psv
