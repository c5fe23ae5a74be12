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
// pairs into FP64 once per gradient. With Step::g_part_lmu set, each step's
// terms first go into FP32 partial sums per point, which the flush steps
// (every few steps, and the last) add into the pairs. There lambda's term
// is folded into the gradients of lm and mu: the FP32 forward forms
// lambda = lm - 2 mu, so d/dlm gains the lambda term and d/dmu loses twice
// it, i.e. t_lm = dt (yxx + yzz)(exx + ezz) and t_mu = dt (yxz gxz -
// 2 (yxx ezz + yzz exx)). Three sums (lm, mu | b) per point: per step the
// kernel reads and writes 12 bytes of sums per point instead of 32 (and
// the pairs of three gradients on flush steps only).
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
static_assert((VB * 4) % 128 == 0 && (SB * 4) % 128 == 0, "boxes must stay 128-byte aligned");
static_assert(TZ == 32 && TX * TZ == 2 * NT, "a pair of own points per thread");

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

__device__ __forceinline__ float2 ld2(const float *p) {
  return *reinterpret_cast<const float2 *>(p);
}
__device__ __forceinline__ void st2(float *p, float2 v) { *reinterpret_cast<float2 *>(p) = v; }

// Staggered differences of a pair of adjacent points k, k + 1 (k even) from
// three float2 loads of their row, L = [k-2, k-1], C = [k, k+1],
// R = [k+2, k+3], with folded coefficients a1 = c1 / h, a2 = c2 / h:
// backward D- f(k) = a1 (f[k] - f[k-1]) + a2 (f[k-2] - f[k+1]),
// forward  D+ f(k) = a1 (f[k+1] - f[k]) + a2 (f[k-1] - f[k+2]).
__device__ __forceinline__ float2 dm_pair(float2 L, float2 C, float2 R, float a1, float a2) {
  return make_float2(a1 * (C.x - L.y) + a2 * (L.x - C.y), a1 * (C.y - C.x) + a2 * (L.y - R.x));
}
__device__ __forceinline__ float2 dp_pair(float2 L, float2 C, float2 R, float a1, float a2) {
  return make_float2(a1 * (C.y - C.x) + a2 * (L.y - R.x), a1 * (R.x - C.y) + a2 * (C.x - R.y));
}
// The same along x from the pair's values in rows -2, -1, 0, +1, +2 (m2 ..
// p2; a row a formula does not use may be anything).
__device__ __forceinline__ float2 dxm_pair(float2 m2, float2 m1, float2 c0, float2 p1, float a1,
                                           float a2) {
  return make_float2(a1 * (c0.x - m1.x) + a2 * (m2.x - p1.x), a1 * (c0.y - m1.y) + a2 * (m2.y - p1.y));
}
__device__ __forceinline__ float2 dxp_pair(float2 m1, float2 c0, float2 p1, float2 p2, float a1,
                                           float a2) {
  return make_float2(a1 * (p1.x - c0.x) + a2 * (m1.x - p2.x), a1 * (p1.y - c0.y) + a2 * (m1.y - p2.y));
}

// Phases 1-3 of one tile (the copies have landed). INNER: every point of
// the 4-halo region is interior with taper 1 and no own point has a source
// term. Phases 2 and 3 give each thread a pair of adjacent z columns: every
// shared-memory access is a float2, and the z-direction stencils of the two
// points share their loads. The difference coefficients are folded with
// 1/dx and 1/dz. Phase 3: thread t owns points (X0 + t / 16,
// Z0 + 2 (t % 16) + {0, 1}); plmu = (lm0, mu0, lm1, mu1) and pb = (b0, b1)
// are their partial sums.
template <bool INNER>
__device__ __forceinline__ void tile_body(const Step &a, float *sm, int X0, int Z0,
                                          float4 plmu, float2 pb) {
  const int tid = threadIdx.x;
  const float c1 = 9.0f / 8.0f, c2 = 1.0f / 24.0f;
  const float c1x = c1 * a.idx, c2x = c2 * a.idx, c1z = c1 * a.idz, c2z = c2 * a.idz;
  const float *LVX = sm + OFF_LV, *LVZ = sm + OFF_LV + VB, *B = sm + OFF_B;
  float *WX = sm + OFF_W, *WZ = sm + OFF_W + VB;
  // Phase 1: w = b dt T lv at interior points, 0 elsewhere.
  if (INNER) {
    static_assert(VB % 4 == 0 && VB / 4 <= NT, "one float4 of the 4-halo box per thread");
    if (tid < VB / 4) {
      const float4 b4 = reinterpret_cast<const float4 *>(B)[tid];
      const float4 x4 = reinterpret_cast<const float4 *>(LVX)[tid];
      const float4 z4 = reinterpret_cast<const float4 *>(LVZ)[tid];
      const float s0 = b4.x * a.dt, s1 = b4.y * a.dt, s2 = b4.z * a.dt, s3 = b4.w * a.dt;
      reinterpret_cast<float4 *>(WX)[tid] = make_float4(s0 * x4.x, s1 * x4.y, s2 * x4.z, s3 * x4.w);
      reinterpret_cast<float4 *>(WZ)[tid] = make_float4(s0 * z4.x, s1 * z4.y, s2 * z4.z, s3 * z4.w);
    }
  } else {
    for (int k = tid; k < VB; k += NT) {
      const int r = k / W, c = k - r * W;
      const int ix = X0 - 4 + r, jz = Z0 - 4 + c;
      float wx = 0.f, wz = 0.f;
      if (ix >= 0 && ix < a.nx && jz >= 0 && jz < a.nz && interior(a, ix, jz)) {
        const float s = B[k] * a.dt * taper_at(a, ix, jz);
        wx = s * LVX[k];
        wz = s * LVZ[k];
      }
      WX[k] = wx;
      WZ[k] = wz;
    }
  }
  __syncthreads();

  float *LXX = sm + OFF_LT, *LZZ = sm + OFF_LT + SB, *LXZ = sm + OFF_LT + 2 * SB;
  const float *LM = sm + OFF_M, *MU = sm + OFF_M + 2 * SB;
  float *PX = sm + OFF_P, *PZ = sm + OFF_P + SB, *QQ = sm + OFF_P + 2 * SB;
  // Phase 2: lt~ = lt - (A^T w terms), and p_x = dt (lm y_xx + la y_zz),
  // p_z = dt (la y_xx + lm y_zz), q = dt mu y_xz with y = T lt~ on I, 0
  // elsewhere; over rows X0-2 .. X0+TX+1 and columns Z0-2 .. Z0+TZ+1, a
  // pair of columns per thread and round.
  constexpr int PP = PC / 2;  // column pairs per row
  for (int k = tid; k < SR * PP; k += NT) {
    const int r = k / PP, c = 2 + 2 * (k - r * PP);
    const int ix = X0 - 2 + r, jz = Z0 - 4 + c;
    const int s = r * W + c;        // in the 2-halo boxes
    const int v = (r + 2) * W + c;  // the same points in the 4-halo boxes
    const float2 wxm1 = ld2(WX + v - W), wx0 = ld2(WX + v), wxp1 = ld2(WX + v + W),
                 wxp2 = ld2(WX + v + 2 * W), wxl = ld2(WX + v - 2), wxr = ld2(WX + v + 2);
    const float2 wzm2 = ld2(WZ + v - 2 * W), wzm1 = ld2(WZ + v - W), wz0 = ld2(WZ + v),
                 wzp1 = ld2(WZ + v + W), wzl = ld2(WZ + v - 2), wzr = ld2(WZ + v + 2);
    const float2 dxp_wx = dxp_pair(wxm1, wx0, wxp1, wxp2, c1x, c2x);
    const float2 dzp_wx = dp_pair(wxl, wx0, wxr, c1z, c2z);
    const float2 dzm_wz = dm_pair(wzl, wz0, wzr, c1z, c2z);
    const float2 dxm_wz = dxm_pair(wzm2, wzm1, wz0, wzp1, c1x, c2x);
    const float2 oxx = ld2(LXX + s), ozz = ld2(LZZ + s), oxz = ld2(LXZ + s);
    float2 lxx = make_float2(oxx.x - dxp_wx.x, oxx.y - dxp_wx.y);
    float2 lzz = make_float2(ozz.x - dzm_wz.x, ozz.y - dzm_wz.y);
    float2 lxz = make_float2(oxz.x - dzp_wx.x - dxm_wz.x, oxz.y - dzp_wx.y - dxm_wz.y);
    const float2 lm = ld2(LM + s), mu = ld2(MU + s);
    float2 px, pz, q;
    if (INNER) {
      const float la0 = lm.x - 2.0f * mu.x, la1 = lm.y - 2.0f * mu.y;
      px = make_float2(a.dt * (lm.x * lxx.x + la0 * lzz.x), a.dt * (lm.y * lxx.y + la1 * lzz.y));
      pz = make_float2(a.dt * (la0 * lxx.x + lm.x * lzz.x), a.dt * (la1 * lxx.y + lm.y * lzz.y));
      q = make_float2(a.dt * mu.x * lxz.x, a.dt * mu.y * lxz.y);
    } else {
      float pxv[2] = {0.f, 0.f}, pzv[2] = {0.f, 0.f}, qv[2] = {0.f, 0.f};
      float lxxv[2] = {lxx.x, lxx.y}, lzzv[2] = {lzz.x, lzz.y}, lxzv[2] = {lxz.x, lxz.y};
      const float oxxv[2] = {oxx.x, oxx.y}, ozzv[2] = {ozz.x, ozz.y}, oxzv[2] = {oxz.x, oxz.y};
      const float lmv[2] = {lm.x, lm.y}, muv[2] = {mu.x, mu.y};
#pragma unroll
      for (int e = 0; e < 2; ++e) {
        const int j = jz + e;
        if (!(ix >= 0 && ix < a.nx && j >= 0 && j < a.nz)) {
          lxxv[e] = oxxv[e];  // outside the grid: lt~ is not formed there
          lzzv[e] = ozzv[e];
          lxzv[e] = oxzv[e];
          continue;
        }
        if (interior(a, ix, j)) {
          const float tp = taper_at(a, ix, j);
          const float yxx = tp * lxxv[e], yzz = tp * lzzv[e], yxz = tp * lxzv[e];
          if (!(yxx == 0.f && yzz == 0.f && yxz == 0.f)) {
            const float la = lmv[e] - 2.0f * muv[e];
            pxv[e] = a.dt * (lmv[e] * yxx + la * yzz);
            pzv[e] = a.dt * (la * yxx + lmv[e] * yzz);
            qv[e] = a.dt * muv[e] * yxz;
          }
        }
      }
      lxx = make_float2(lxxv[0], lxxv[1]);
      lzz = make_float2(lzzv[0], lzzv[1]);
      lxz = make_float2(lxzv[0], lxzv[1]);
      px = make_float2(pxv[0], pxv[1]);
      pz = make_float2(pzv[0], pzv[1]);
      q = make_float2(qv[0], qv[1]);
    }
    st2(LXX + s, lxx);
    st2(LZZ + s, lzz);
    st2(LXZ + s, lxz);
    st2(PX + s, px);
    st2(PZ + s, pz);
    st2(QQ + s, q);
  }
  __syncthreads();

  // Phase 3: own points, a pair per thread.
  const int lx = tid >> 4, c = 4 + 2 * (tid & 15);
  const int ix = X0 + lx, iz = Z0 + c - 4;
  if (!INNER && (ix >= a.nx || iz >= a.nz)) return;
  const float *FVX = sm + OFF_FV, *FVZ = sm + OFF_FV + SB;
  const float *FXX = sm + OFF_FT, *FZZ = sm + OFF_FT + SB, *FXZ = sm + OFF_FT + 2 * SB;
  const int tile = blockIdx.x;
  const int r0 = a.rec_start[tile], r1 = a.rec_start[tile + 1];
  const int s = (lx + 2) * W + c;  // 2-halo boxes
  const int v = (lx + 4) * W + c;  // 4-halo boxes
  const float2 lxx = ld2(LXX + s), lzz = ld2(LZZ + s), lxz = ld2(LXZ + s);
  const float2 lvx = ld2(LVX + v), lvz = ld2(LVZ + v);
  const bool part = a.g_part_lmu != nullptr;
  const float lxxv[2] = {lxx.x, lxx.y}, lzzv[2] = {lzz.x, lzz.y}, lxzv[2] = {lxz.x, lxz.y};
  const float lvxv[2] = {lvx.x, lvx.y}, lvzv[2] = {lvz.x, lvz.y};
  // Per point: inside the grid, interior, taper.
  bool validv[2], inv[2];
  float tpv[2];
#pragma unroll
  for (int e = 0; e < 2; ++e) {
    validv[e] = INNER || iz + e < a.nz;
    inv[e] = INNER || (validv[e] && interior(a, ix, iz + e));
    tpv[e] = (INNER || !inv[e]) ? 1.f : taper_at(a, ix, iz + e);
  }
  const size_t p0 = (size_t)ix * a.pitch + iz;
  const bool both = INNER || iz + 1 < a.nz;
  // Stage 1: the adjoint state. tau-bar^n = T lt~;
  // E^T (dt C y):  v-bar_x += -D-_x(p_x)/dx - D-_z(q)/dz,
  //                v-bar_z += -D+_z(p_z)/dz - D+_x(q)/dx
  {
    const float2 dxm_px = dxm_pair(ld2(PX + s - 2 * W), ld2(PX + s - W), ld2(PX + s),
                                   ld2(PX + s + W), c1x, c2x);
    const float2 q0 = ld2(QQ + s);
    const float2 dzm_q = dm_pair(ld2(QQ + s - 2), q0, ld2(QQ + s + 2), c1z, c2z);
    const float2 dxp_q =
        dxp_pair(ld2(QQ + s - W), q0, ld2(QQ + s + W), ld2(QQ + s + 2 * W), c1x, c2x);
    const float2 dzp_pz = dp_pair(ld2(PZ + s - 2), ld2(PZ + s), ld2(PZ + s + 2), c1z, c2z);
    float ovx[2] = {tpv[0] * lvx.x - dxm_px.x - dzm_q.x, tpv[1] * lvx.y - dxm_px.y - dzm_q.y};
    float ovz[2] = {tpv[0] * lvz.x - dzp_pz.x - dxp_q.x, tpv[1] * lvz.y - dzp_pz.y - dxp_q.y};
    // Receiver terms v-bar^n(rec) += adj[r][n].
    for (int i = r0; i < r1; ++i) {
      const int rr = a.rec_list[i];
      const int cell = a.rec_cell[rr];
#pragma unroll
      for (int e = 0; e < 2; ++e)
        if (cell == (int)(p0 + e)) {
          ovx[e] = ovx[e] + (float)a.adj_x[(size_t)rr * a.nt + a.it];
          ovz[e] = ovz[e] + (float)a.adj_z[(size_t)rr * a.nt + a.it];
        }
    }
    if (both) {
      st2(a.olt[0] + p0, make_float2(tpv[0] * lxx.x, tpv[1] * lxx.y));
      st2(a.olt[1] + p0, make_float2(tpv[0] * lzz.x, tpv[1] * lzz.y));
      st2(a.olt[2] + p0, make_float2(tpv[0] * lxz.x, tpv[1] * lxz.y));
      st2(a.olv[0] + p0, make_float2(ovx[0], ovx[1]));
      st2(a.olv[1] + p0, make_float2(ovz[0], ovz[1]));
    } else {
      a.olt[0][p0] = tpv[0] * lxx.x;
      a.olt[1][p0] = tpv[0] * lzz.x;
      a.olt[2][p0] = tpv[0] * lxz.x;
      a.olv[0][p0] = ovx[0];
      a.olv[1][p0] = ovz[0];
    }
  }
  // Stage 2: the gradient terms: grad_b += dt T lv . A tau^{n+1}, medium
  // gradients from the strain rates of v^n.
  const float2 fxz0 = ld2(FXZ + s);
  const float2 ax_x = dxm_pair(ld2(FXX + s - 2 * W), ld2(FXX + s - W), ld2(FXX + s),
                               ld2(FXX + s + W), c1x, c2x);
  const float2 ax_z = dm_pair(ld2(FXZ + s - 2), fxz0, ld2(FXZ + s + 2), c1z, c2z);
  const float2 az_x = dxp_pair(ld2(FXZ + s - W), fxz0, ld2(FXZ + s + W), ld2(FXZ + s + 2 * W),
                               c1x, c2x);
  const float2 az_z = dp_pair(ld2(FZZ + s - 2), ld2(FZZ + s), ld2(FZZ + s + 2), c1z, c2z);
  const float axv[2] = {ax_x.x + ax_z.x, ax_x.y + ax_z.y};
  const float azv[2] = {az_x.x + az_z.x, az_x.y + az_z.y};
  const float2 fvx0 = ld2(FVX + s), fvz0 = ld2(FVZ + s);
  const float2 ex = dxp_pair(ld2(FVX + s - W), fvx0, ld2(FVX + s + W), ld2(FVX + s + 2 * W), c1x,
                             c2x);
  const float2 gxz_x = dp_pair(ld2(FVX + s - 2), fvx0, ld2(FVX + s + 2), c1z, c2z);
  const float2 ez = dm_pair(ld2(FVZ + s - 2), fvz0, ld2(FVZ + s + 2), c1z, c2z);
  const float2 gxz_z = dxm_pair(ld2(FVZ + s - 2 * W), ld2(FVZ + s - W), fvz0, ld2(FVZ + s + W),
                                c1x, c2x);
  const float exv[2] = {ex.x, ex.y}, ezv[2] = {ez.x, ez.y};
  const float gxzv[2] = {gxz_x.x + gxz_z.x, gxz_x.y + gxz_z.y};
  float pl_lm[2] = {plmu.x, plmu.z}, pl_mu[2] = {plmu.y, plmu.w}, pl_b[2] = {pb.x, pb.y};
#pragma unroll
  for (int e = 0; e < 2; ++e) {
    if (!validv[e]) continue;
    const int jz = iz + e;
    const size_t u = (size_t)ix * a.nz + jz;
    const float tp = tpv[e];
    // The float-float pairs, where this step adds into them.
    float2 glm = make_float2(0.f, 0.f), gla = glm, gmu = glm, g_b = glm;
    if (!part || a.flush) {
      glm = a.g_lm[u];
      if (!part) gla = a.g_la[u];
      gmu = a.g_mu[u];
      g_b = a.g_b[u];
    }
    float t_lm = 0.f, t_mu = 0.f, t_b = 0.f;
    if (inv[e]) {
      t_b = (a.dt * tp) * (lvxv[e] * axv[e] + lvzv[e] * azv[e]);
      const float yxx = tp * lxxv[e], yzz = tp * lzzv[e], yxz = tp * lxzv[e];
      if (!part) {
        g_b = ff_add(g_b, t_b);
        a.g_lm[u] = ff_add(glm, a.dt * (yxx * exv[e] + yzz * ezv[e]));
        a.g_la[u] = ff_add(gla, a.dt * (yxx * ezv[e] + yzz * exv[e]));
        a.g_mu[u] = ff_add(gmu, a.dt * yxz * gxzv[e]);
      } else {
        t_lm = a.dt * ((yxx + yzz) * (exv[e] + ezv[e]));
        t_mu = a.dt * (yxz * gxzv[e] - 2.f * (yxx * ezv[e] + yzz * exv[e]));
      }
    }
    // Source terms s = coef stf dt b / div at their points depend on b.
    const InjPlan &pl = a.plan;
    bool src = false;
    if (!INNER && pl.n && ix >= pl.x0 && ix < pl.x0 + pl.w && jz >= pl.z0 && jz < pl.z0 + pl.h) {
      int k = pl.map[(ix - pl.x0) * pl.h + (jz - pl.z0)];
      for (; k >= 0 && k < pl.n && pl.terms[k].cell == (int)u; ++k) {
        const InjTerm t = pl.terms[k];
        if (t.kind != 0) continue;
        const double ds = ((t.coef * a.stf[(size_t)t.index * a.nt + a.it]) * a.dt_d) / t.div;
        const float ts = (float)(ds * (double)(t.field == 0 ? lvxv[e] : lvzv[e]));
        if (part)
          t_b += ts;
        else
          g_b = ff_add(g_b, ts);
        src = true;
      }
    }
    if (!part) {
      if (inv[e] || src) a.g_b[u] = g_b;
      continue;
    }
    pl_lm[e] += t_lm;
    pl_mu[e] += t_mu;
    pl_b[e] += t_b;
    if (a.flush) {
      a.g_lm[u] = ff_add(glm, pl_lm[e]);
      a.g_mu[u] = ff_add(gmu, pl_mu[e]);
      a.g_b[u] = ff_add(g_b, pl_b[e]);
      pl_lm[e] = pl_mu[e] = pl_b[e] = 0.f;
    }
  }
  // The pair's partial sums (the second point may be row padding, where
  // the sums stay 0).
  if (part && validv[0]) {
    const size_t q = (size_t)ix * a.pitch + iz;
    reinterpret_cast<float4 *>(a.g_part_lmu + q)[0] =
        make_float4(pl_lm[0], pl_mu[0], pl_lm[1], pl_mu[1]);
    reinterpret_cast<float2 *>(a.g_part_b + q)[0] = make_float2(pl_b[0], pl_b[1]);
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

  // This thread's own points (row X0 + tid / 16, columns Z0 + 2 (tid % 16)
  // + {0, 1}) and their gradient sums, loaded while the copies fly.
  // (With partial sums, the pairs are read only on flush steps.)
  // (The float-float pairs are read in phase 3, where they are needed:
  // every step without partial sums, flush steps with them.)
  // The pair's sums are adjacent in the padded rows (own_z is even and the
  // pitch a multiple of 4), so they load as one float4 and one float2.
  float4 plmu = make_float4(0.f, 0.f, 0.f, 0.f);
  float2 pb = make_float2(0.f, 0.f);
  const int own_x = X0 + (tid >> 4), own_z = Z0 + 2 * (tid & 15);
  if (a.g_part_lmu && own_x < a.nx && own_z < a.nz) {
    const size_t q = (size_t)own_x * a.pitch + own_z;
    plmu = reinterpret_cast<const float4 *>(a.g_part_lmu + q)[0];
    pb = reinterpret_cast<const float2 *>(a.g_part_b + q)[0];
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
    tile_body<true>(a, sm, X0, Z0, plmu, pb);
  else
    tile_body<false>(a, sm, X0, Z0, plmu, pb);
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
