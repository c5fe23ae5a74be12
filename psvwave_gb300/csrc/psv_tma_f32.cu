// FP32 fused time step with TMA tile loads, for a table of simulations.
//
// Each CTA owns a TX x TZ tile of one simulation (one shot of one model).
// Thread 0 issues seven cp.async.bulk.tensor.2d loads -- vx, vz with a
// 4-point halo; txx, tzz, txz, lm, mu with a 2-point halo -- completing on
// one mbarrier; the copies zero-fill whatever lies outside the grid. The CTA
// then advances the stresses over the tile plus a 2-point halo in shared
// memory (halo points are recomputed by the neighbours too), and finishes
// with the new velocities of its own points. Old and new wave fields live in
// separate buffer sets (ping-pong), so one launch per time step covers all
// simulations without any grid-wide barrier. lambda is lm - 2 mu.
//
// Arithmetic: the reference's stencil (src/fdModel.cpp:599-678 forward,
// 864-948 adjoint) in float with reciprocal multiplies; snapshot storage
// (src/fdModel.cpp:555-572), kernel correlation (src/fdModel.cpp:817-861,
// FP64 accumulation), receiver sampling (src/fdModel.cpp:576-596) and source
// / adjoint-source injection (src/fdModel.cpp:681-751, 951-958) are fused in.
//
// A TMA copy must start on a 16-byte boundary of the innermost (z) axis:
// every box starts at z = Z0 - 4 with Z0 a multiple of TZ (TZ a multiple of
// 4) and is TZ + 8 points wide; rows are padded to a multiple of 4 points.
// Warps of the compute phases own 32 consecutive z columns. Three kinds of
// tile take three paths: interior tiles (taper exactly 1, no per-point
// tests) and, on the 128-thread shapes, taper tiles (inside the updated
// region, in the absorbing frame) walk consecutive rows with the x-direction
// stencil values in registers; the others walk every G-th row with
// per-point bounds and taper tests. Tile shapes: 32 x 60 (256 threads),
// 16 x 28 and 20 x 28 (128 threads).
//
// Launch schemes: one launch per time step (fused_step_tma, and
// fused_step_tma_batch over a tile table), or every step in one persistent
// cooperative launch (fused_steps_tma, fused_steps_tma_batch) whose CTAs
// take (step, tile) items in step order, start an item once the tile and
// its neighbours have published the previous step, and publish with a
// barrier plus one release store.
//
// Every wait is bounded: on time-out the CTA raises the error flag, waits
// (bounded again) for its copies to land, and returns.
#include <cuda.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>

#include "psv_tma.hpp"
#include "psv_tma_ptx.cuh"
#include "psv_tma_terms.cuh"

namespace psv {
namespace tma {
namespace {

template <int TX_, int TZ_, int NT_, int MINB_>
struct Shape {
  static constexpr int TX = TX_, TZ = TZ_, NT = NT_;
  static constexpr int MINB = MINB_;  // resident CTAs per SM the registers must allow
  static constexpr int W = TZ + 8;    // box width (z): Z0-4 .. Z0+TZ+4
  static constexpr int VR = TX + 8;   // velocity box rows: X0-4 .. X0+TX+4
  static constexpr int SR = TX + 4;   // stress / medium box rows: X0-2 .. X0+TX+2
  static constexpr int SC = TZ + 4;   // stress columns computed (box columns 2 .. TZ+6)
  static constexpr int WARPS = NT / 32;
  static constexpr int H = SC / 32;       // warps across the columns
  static constexpr int G = WARPS / H;     // row groups
  static constexpr int VBYTES = VR * W * 4;
  static constexpr int SBYTES = SR * W * 4;
  static constexpr int SPITCH = (SBYTES + 127) / 128 * 128;
  static constexpr int VPITCH = (VBYTES + 127) / 128 * 128;
  static constexpr int TX_BYTES = 2 * VBYTES + 5 * SBYTES;  // delivered by the copies
  static constexpr int TILE_BYTES = 2 * VPITCH + 5 * SPITCH;
  static constexpr int SMEM = TILE_BYTES + 16 + 128;        // + mbarrier + alignment slack
  static_assert(SC % 32 == 0, "warps must span the stress columns");
  static_assert(WARPS % H == 0 && SR % G == 0 && TX % G == 0, "row groups must tile the rows");
  static_assert(TZ % 4 == 0, "tile columns must keep TMA boxes 16-byte aligned");
};
using Big = Shape<32, 60, 256, 3>;
using Small = Shape<16, 28, 128, 8>;
using Mid = Shape<20, 28, 128, 8>;
using Wide = Shape<16, 60, 128, 5>;

// Calls f with the shape type and its TileCfg value for `cfg`.
template <class S_, int CFG_>
struct ShapeTag {
  using S = S_;
  static constexpr int CFG = CFG_;
};
template <class F>
decltype(auto) with_shape(int cfg, F &&f) {
  if (cfg == kTile16x28) return f(ShapeTag<Small, kTile16x28>{});
  if (cfg == kTile20x28) return f(ShapeTag<Mid, kTile20x28>{});
  if (cfg == kTile16x60) return f(ShapeTag<Wide, kTile16x60>{});
  return f(ShapeTag<Big, kTile32x60>{});
}

// A call made between phase B and phase C of a tile (the persistent step
// draws its next item there).
struct NoHook {
  __device__ void operator()() const {}
};

// An interior tile computes every stress point of its box (rows X0-2 ..
// X0+TX+1, columns Z0-2 .. Z0+TZ+1) inside the updated region 2 <= x < n-2
// and at least np frames deep (taper exactly 1), has no source or
// adjoint-source term among its own points and no snapshot I/O this step.
// Its copies then lie wholly inside the grid and it needs no per-point test.
template <class S>
__device__ __forceinline__ bool interior_tile(const SimDesc &d, int X0, int Z0, bool snap_io) {
  const int lo = max(2, d.np - 1);
  const InjPlan &p = d.plan;
  const bool inj = p.n && X0 < p.x0 + p.w && p.x0 < X0 + S::TX && Z0 < p.z0 + p.h &&
                   p.z0 < Z0 + S::TZ;
  return !snap_io && !inj && X0 - 2 >= lo && Z0 - 2 >= lo &&
         X0 + S::TX + 1 <= min(d.nx - 3, d.nx - d.np) &&
         Z0 + S::TZ + 1 <= min(d.nz - 3, d.nz - d.np);
}

// A taper tile has every stress point of its box inside the updated region
// but lies (partly) in the absorbing frame; no source or snapshot I/O. It
// takes the interior path with the taper factor applied.
template <class S>
__device__ __forceinline__ bool taper_tile(const SimDesc &d, int X0, int Z0, bool snap_io) {
  const InjPlan &p = d.plan;
  const bool inj = p.n && X0 < p.x0 + p.w && p.x0 < X0 + S::TX && Z0 < p.z0 + p.h &&
                   p.z0 < Z0 + S::TZ;
  return !snap_io && !inj && X0 - 2 >= 2 && Z0 - 2 >= 2 && X0 + S::TX + 1 <= d.nx - 3 &&
         Z0 + S::TZ + 1 <= d.nz - 3;
}

// Taper factor of grid point (gx, gz) from the column factor tzc: the table
// at the point's frame count min(tz, tx) (1 from np frames on) is the
// smaller of the table at tz and at tx, since the Cerjan taper grows with
// the count.
__device__ __forceinline__ float row_taper(const SimDesc &d, int gx) {
  const int tx = min(gx + 1, d.nx - gx);
  return tx < d.np ? __ldg(d.taper_tab + tx) : 1.0f;
}
__device__ __forceinline__ float col_taper(const SimDesc &d, int gz) {
  const int tz = min(gz + 1, d.nz - gz);
  return tz < d.np ? __ldg(d.taper_tab + tz) : 1.0f;
}

// Frame-count taper of a row or column at grid index g of an n-point axis,
// for any g (points outside the grid clamp to the table's first entry; their
// updates are masked out).
__device__ __forceinline__ float axis_taper(const SimDesc &d, int g, int n) {
  const int t = max(min(g + 1, n - g), 0);
  return t < d.np ? __ldg(d.taper_tab + t) : 1.0f;
}

// Phases B and C of an interior tile (TAPER false: taper exactly 1), a
// taper tile (TAPER true) or a frame tile of a one-column shape (FRAME true:
// the box may reach past the grid's edges; per-point taper min(column
// factor, row factor) and masks that keep points outside the updated region
// 2 <= x < n-2 at their old values, and own points past the grid unwritten).
// Phase B: each thread walks SR / G consecutive rows of one column, keeping
// the x-direction stencil values of vx and vz in registers (one new shared
// load each per row); phase C: KC consecutive rows per thread with the
// x-direction windows of txx and txz.
template <class S, bool ADJ, bool TAPER, bool FRAME = false, class Mid = NoHook>
__device__ __forceinline__ void tile_phases(const SimDesc &d, const fast::Fields &out, int X0,
                                            int Z0, const float (*VX)[S::W],
                                            const float (*VZ)[S::W], float (*sxx_)[S::W],
                                            float (*szz_)[S::W], float (*sxz_)[S::W],
                                            const float (*slm)[S::W], const float (*smu)[S::W],
                                            const float *bb, const Mid &mid = Mid()) {
  constexpr int TX = S::TX, TZ = S::TZ, SR = S::SR, G = S::G;
  constexpr int KC = TX / G;
  const int ps = d.pitch;
  const float c1 = 9.0f / 8.0f, c2 = 1.0f / 24.0f;
  const float dtv = ADJ ? -d.dt : d.dt;
  const float idx = d.idx, idz = d.idz;
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, h = w % S::H, q = w / S::H;
  const int lzc = h * 32 + lane;
  const int gzc = Z0 + lzc;
  {
    constexpr int RB = SR / G;
    const int c = 2 + h * 32 + lane;
    const int gz = Z0 - 4 + c;
    const bool z_own = c >= 4 && c < TZ + 4;
    const int r0 = q * RB;
    const float tzc = FRAME ? axis_taper(d, gz, d.nz) : TAPER ? col_taper(d, gz) : 1.0f;
    const bool zi = !FRAME || (gz >= 2 && gz < d.nz - 2);
    const bool z_out = !FRAME || gz < d.nz;
    float xm1 = VX[r0 + 1][c], x0 = VX[r0 + 2][c], xp1 = VX[r0 + 3][c], xp2 = VX[r0 + 4][c];
    float zm2 = VZ[r0][c], zm1 = VZ[r0 + 1][c], z0 = VZ[r0 + 2][c], zp1 = VZ[r0 + 3][c];
    int gp = (X0 - 2 + r0) * ps + gz;
#pragma unroll
    for (int k = 0; k < RB; ++k) {
      const int r = r0 + k, vr = r + 2;
      const float lm = slm[r][c], mu = smu[r][c];
      const float la = lm - 2.0f * mu;
      const float dvx = c1 * (xp1 - x0) + c2 * (xm1 - xp2);
      const float dvz = c1 * (z0 - VZ[vr][c - 1]) + c2 * (VZ[vr][c - 2] - VZ[vr][c + 1]);
      const float gxz = (c1 * (VX[vr][c + 1] - x0) + c2 * (VX[vr][c - 1] - VX[vr][c + 2])) * idz +
                        (c1 * (z0 - zm1) + c2 * (zm2 - zp1)) * idx;
      const float ex = dvx * idx, ez = dvz * idz;
      float sxx, szz, sxz;
      if (FRAME) {
        const int gx = X0 - 2 + r;
        const float tp = fminf(tzc, axis_taper(d, gx, d.nx));
        const bool u = zi && gx >= 2 && gx < d.nx - 2;
        const float oxx = sxx_[r][c], ozz = szz_[r][c], oxz = sxz_[r][c];
        sxx = u ? tp * (oxx + dtv * (lm * ex + la * ez)) : oxx;
        szz = u ? tp * (ozz + dtv * (la * ex + lm * ez)) : ozz;
        sxz = u ? tp * (oxz + dtv * mu * gxz) : oxz;
      } else if (TAPER) {
        const float tp = fminf(tzc, row_taper(d, X0 - 2 + r));
        sxx = tp * (sxx_[r][c] + dtv * (lm * ex + la * ez));
        szz = tp * (szz_[r][c] + dtv * (la * ex + lm * ez));
        sxz = tp * (sxz_[r][c] + dtv * mu * gxz);
      } else {
        sxx = sxx_[r][c] + dtv * (lm * ex + la * ez);
        szz = szz_[r][c] + dtv * (la * ex + lm * ez);
        sxz = sxz_[r][c] + dtv * mu * gxz;
      }
      sxx_[r][c] = sxx;
      szz_[r][c] = szz;
      sxz_[r][c] = sxz;
      if (z_own && r >= 2 && r < TX + 2 && z_out && (!FRAME || X0 - 2 + r < d.nx)) {
        out.txx[gp] = sxx;
        out.tzz[gp] = szz;
        out.txz[gp] = sxz;
      }
      gp += ps;
      if (k + 1 < RB) {
        xm1 = x0;
        x0 = xp1;
        xp1 = xp2;
        xp2 = VX[vr + 3][c];
        zm2 = zm1;
        zm1 = z0;
        z0 = zp1;
        zp1 = VZ[vr + 2][c];
      }
    }
  }
  __syncthreads();
  mid();
  if (lzc < TZ) {
    const float(*TXX)[S::W] = sxx_;
    const float(*TZZ)[S::W] = szz_;
    const float(*TXZ)[S::W] = sxz_;
    const int cc = lzc + 4;
    const int lx0 = q * KC;
    const int s0 = lx0 + 2;  // stress box row of the first point
    const float tzc = FRAME ? axis_taper(d, gzc, d.nz) : TAPER ? col_taper(d, gzc) : 1.0f;
    const bool zi = !FRAME || (gzc >= 2 && gzc < d.nz - 2);
    const bool z_out = !FRAME || gzc < d.nz;
    float am2 = TXX[s0 - 2][cc], am1 = TXX[s0 - 1][cc], a0 = TXX[s0][cc], ap1 = TXX[s0 + 1][cc];
    float bm1 = TXZ[s0 - 1][cc], b0 = TXZ[s0][cc], bp1 = TXZ[s0 + 1][cc], bp2 = TXZ[s0 + 2][cc];
    int gq = (X0 + lx0) * ps + gzc;
#pragma unroll
    for (int k = 0; k < KC; ++k) {
      const int r = s0 + k, lx = lx0 + k;
      const float ax = (c1 * (a0 - am1) + c2 * (am2 - ap1)) * idx +
                       (c1 * (b0 - TXZ[r][cc - 1]) + c2 * (TXZ[r][cc - 2] - TXZ[r][cc + 1])) * idz;
      const float az = (c1 * (bp1 - b0) + c2 * (bm1 - bp2)) * idx +
                       (c1 * (TZZ[r][cc + 1] - TZZ[r][cc]) + c2 * (TZZ[r][cc - 1] - TZZ[r][cc + 2])) * idz;
      const float bdt = bb[k] * dtv;
      if (FRAME) {
        const int gx = X0 + lx;
        const float tp = fminf(tzc, axis_taper(d, gx, d.nx));
        const bool u = zi && gx >= 2 && gx < d.nx - 2;
        const float ovx = VX[lx + 4][cc], ovz = VZ[lx + 4][cc];
        if (z_out && gx < d.nx) {
          out.vx[gq] = u ? tp * (ovx + bdt * ax) : ovx;
          out.vz[gq] = u ? tp * (ovz + bdt * az) : ovz;
        }
      } else if (TAPER) {
        const float tp = fminf(tzc, row_taper(d, X0 + lx));
        out.vx[gq] = tp * (VX[lx + 4][cc] + bdt * ax);
        out.vz[gq] = tp * (VZ[lx + 4][cc] + bdt * az);
      } else {
        out.vx[gq] = VX[lx + 4][cc] + bdt * ax;
        out.vz[gq] = VZ[lx + 4][cc] + bdt * az;
      }
      gq += ps;
      if (k + 1 < KC) {
        am2 = am1;
        am1 = a0;
        a0 = ap1;
        ap1 = TXX[r + 2][cc];
        bm1 = b0;
        b0 = bp1;
        bp1 = bp2;
        bp2 = TXZ[r + 3][cc];
      }
    }
  }
}

// A frame tile has no snapshot I/O this step, no injection term, and its own
// columns lie inside the grid (its own rows may end at the grid's last row;
// its halo may lie outside). It takes the vectorised path with per-point
// taper factors and masks that keep points outside the updated region
// 2 <= x < n-2 at their old values. (Injection tiles keep the one-column
// path: there each thread adds the terms of at most a few points, whose
// dependent loads of the plan and wavelet are the tile's critical path;
// with two columns and four rows per thread that chain grew so long that
// the source tile held back its neighbours' steps.)
template <class S>
__device__ __forceinline__ bool injection_tile(const SimDesc &d, int X0, int Z0) {
  const InjPlan &p = d.plan;
  return p.n && X0 < p.x0 + p.w && p.x0 < X0 + S::TX && Z0 < p.z0 + p.h && p.z0 < Z0 + S::TZ;
}
template <class S>
__device__ __forceinline__ bool frame_tile(const SimDesc &d, int X0, int Z0, bool snap_io) {
  return !snap_io && Z0 + S::TZ <= d.nz && !injection_tile<S>(d, X0, Z0);
}

__device__ __forceinline__ float2 lds2(const float *p) {
  return *reinterpret_cast<const float2 *>(p);
}
__device__ __forceinline__ void sts2(float *p, float2 v) { *reinterpret_cast<float2 *>(p) = v; }

// Phases B and C of the 60-column shapes (32 x 60, 16 x 60) with two z
// columns per lane: every shared-memory access is a float2 (the z-direction
// stencil of two adjacent points shares its loads), each warp walks
// consecutive rows with the x-direction stencil values in registers, and the
// difference coefficients are folded with 1/dx and 1/dz. Phase B: a warp
// covers the 64 stress columns and RQ or RQ + 1 of the TX + 4 rows (32 x 60:
// warps 0-3 five and 4-7 four of 36; 16 x 60: five each of 20); phase C:
// lanes 0-29 cover the 60 own columns, each warp KV = TX / warps own rows.
// FRAME false: an interior tile (taper exactly 1, every point updated);
// FRAME true: a frame tile (taper = min of the row and column factors, which
// is the table at the point's frame count because the Cerjan taper grows
// with the count; points outside the updated region keep their values; own
// rows beyond the grid's last row are skipped).
// bb: this thread's buoyancy, rows X0 + KV w + k (KV = TX / warps own rows
// per warp), columns Z0 + 2 lane + {0,1}.
template <class S, bool ADJ, bool FRAME, class Mid = NoHook>
__device__ __forceinline__ void tile_phases_v2(const SimDesc &d, const fast::Fields &out, int X0,
                                               int Z0, const float (*VX)[S::W],
                                               const float (*VZ)[S::W], float (*sxx_)[S::W],
                                               float (*szz_)[S::W], float (*sxz_)[S::W],
                                               const float (*slm)[S::W], const float (*smu)[S::W],
                                               const float *bb, const Mid &mid = Mid()) {
  static_assert(S::TZ == 60, "two columns per lane over the 64 stress columns");
  constexpr int TX = S::TX, TZ = S::TZ, WARPS = S::WARPS, SR = S::SR;
  // Stress rows: warp w takes RQ or RQ + 1 consecutive rows; own rows: KV.
  constexpr int RQ = SR / WARPS, RR = SR % WARPS, RB = RQ + (RR ? 1 : 0), KV = TX / WARPS;
  static_assert(TX % WARPS == 0, "own rows split evenly over the warps");
  const int ps = d.pitch, nx = d.nx, nz = d.nz;
  const float dtv = ADJ ? -d.dt : d.dt;
  const float c1x = (9.0f / 8.0f) * d.idx, c2x = (1.0f / 24.0f) * d.idx;
  const float c1z = (9.0f / 8.0f) * d.idz, c2z = (1.0f / 24.0f) * d.idz;
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  {
    const int c = 2 + 2 * lane;  // box columns c, c + 1
    const int gz = Z0 - 4 + c;
    const bool z_own = c >= 4 && c < TZ + 4;
    const int r0 = w * RQ + min(w, RR);
    const int nr = RQ + (w < RR ? 1 : 0);
    float tz0 = 1.0f, tz1 = 1.0f;
    bool zi0 = true, zi1 = true;
    if (FRAME) {
      tz0 = axis_taper(d, gz, nz);
      tz1 = axis_taper(d, gz + 1, nz);
      zi0 = gz >= 2 && gz < nz - 2;
      zi1 = gz + 1 >= 2 && gz + 1 < nz - 2;
    }
    float2 xm1 = lds2(&VX[r0 + 1][c]), x0 = lds2(&VX[r0 + 2][c]), xp1 = lds2(&VX[r0 + 3][c]),
           xp2 = lds2(&VX[r0 + 4][c]);
    float2 zm2 = lds2(&VZ[r0][c]), zm1 = lds2(&VZ[r0 + 1][c]), z0 = lds2(&VZ[r0 + 2][c]),
           zp1 = lds2(&VZ[r0 + 3][c]);
    int gp = (X0 - 2 + r0) * ps + gz;
#pragma unroll
    for (int k = 0; k < RB; ++k) {
      if (k < nr) {
        const int r = r0 + k, vr = r + 2;
        const float2 lm = lds2(&slm[r][c]), mu = lds2(&smu[r][c]);
        const float2 vxl = lds2(&VX[vr][c - 2]), vxr = lds2(&VX[vr][c + 2]);
        const float2 vzl = lds2(&VZ[vr][c - 2]), vzr = lds2(&VZ[vr][c + 2]);
        float2 sxx = lds2(&sxx_[r][c]), szz = lds2(&szz_[r][c]), sxz = lds2(&sxz_[r][c]);
        const float ex0 = c1x * (xp1.x - x0.x) + c2x * (xm1.x - xp2.x);
        const float ex1 = c1x * (xp1.y - x0.y) + c2x * (xm1.y - xp2.y);
        const float ez0 = c1z * (z0.x - vzl.y) + c2z * (vzl.x - z0.y);
        const float ez1 = c1z * (z0.y - z0.x) + c2z * (vzl.y - vzr.x);
        const float g0 = (c1z * (x0.y - x0.x) + c2z * (vxl.y - vxr.x)) +
                         (c1x * (z0.x - zm1.x) + c2x * (zm2.x - zp1.x));
        const float g1 = (c1z * (vxr.x - x0.y) + c2z * (x0.x - vxr.y)) +
                         (c1x * (z0.y - zm1.y) + c2x * (zm2.y - zp1.y));
        const float la0 = lm.x - 2.0f * mu.x, la1 = lm.y - 2.0f * mu.y;
        float nxx0 = sxx.x + dtv * (lm.x * ex0 + la0 * ez0);
        float nxx1 = sxx.y + dtv * (lm.y * ex1 + la1 * ez1);
        float nzz0 = szz.x + dtv * (la0 * ex0 + lm.x * ez0);
        float nzz1 = szz.y + dtv * (la1 * ex1 + lm.y * ez1);
        float nxz0 = sxz.x + dtv * mu.x * g0;
        float nxz1 = sxz.y + dtv * mu.y * g1;
        if (FRAME) {
          const int gx = X0 - 2 + r;
          const bool xi = gx >= 2 && gx < nx - 2;
          const float tr = axis_taper(d, gx, nx);
          const float t0 = fminf(tz0, tr), t1 = fminf(tz1, tr);
          const bool u0 = xi && zi0, u1 = xi && zi1;
          sxx.x = u0 ? t0 * nxx0 : sxx.x;
          szz.x = u0 ? t0 * nzz0 : szz.x;
          sxz.x = u0 ? t0 * nxz0 : sxz.x;
          sxx.y = u1 ? t1 * nxx1 : sxx.y;
          szz.y = u1 ? t1 * nzz1 : szz.y;
          sxz.y = u1 ? t1 * nxz1 : sxz.y;
        } else {
          sxx = make_float2(nxx0, nxx1);
          szz = make_float2(nzz0, nzz1);
          sxz = make_float2(nxz0, nxz1);
        }
        sts2(&sxx_[r][c], sxx);
        sts2(&szz_[r][c], szz);
        sts2(&sxz_[r][c], sxz);
        if (z_own && r >= 2 && r < TX + 2 && (!FRAME || X0 - 2 + r < nx)) {
          sts2(out.txx + gp, sxx);
          sts2(out.tzz + gp, szz);
          sts2(out.txz + gp, sxz);
        }
        gp += ps;
        if (k + 1 < nr) {
          xm1 = x0;
          x0 = xp1;
          xp1 = xp2;
          xp2 = lds2(&VX[vr + 3][c]);
          zm2 = zm1;
          zm1 = z0;
          z0 = zp1;
          zp1 = lds2(&VZ[vr + 2][c]);
        }
      }
    }
  }
  __syncthreads();
  mid();
  if (lane < TZ / 2) {
    const float(*TXX)[S::W] = sxx_;
    const float(*TZZ)[S::W] = szz_;
    const float(*TXZ)[S::W] = sxz_;
    const int cc = 4 + 2 * lane;  // box columns cc, cc + 1
    const int gz = Z0 + 2 * lane;
    const int lx0 = KV * w;
    const int s0 = lx0 + 2;  // stress box row of the first point
    float tz0 = 1.0f, tz1 = 1.0f;
    bool zi0 = true, zi1 = true;
    if (FRAME) {
      tz0 = axis_taper(d, gz, nz);
      tz1 = axis_taper(d, gz + 1, nz);
      zi0 = gz >= 2 && gz < nz - 2;
      zi1 = gz + 1 >= 2 && gz + 1 < nz - 2;
    }
    float2 am2 = lds2(&TXX[s0 - 2][cc]), am1 = lds2(&TXX[s0 - 1][cc]), a0 = lds2(&TXX[s0][cc]),
           ap1 = lds2(&TXX[s0 + 1][cc]);
    float2 bm1 = lds2(&TXZ[s0 - 1][cc]), b0 = lds2(&TXZ[s0][cc]), bp1 = lds2(&TXZ[s0 + 1][cc]),
           bp2 = lds2(&TXZ[s0 + 2][cc]);
    int gq = (X0 + lx0) * ps + gz;
#pragma unroll
    for (int k = 0; k < KV; ++k) {
      const int r = s0 + k, lx = lx0 + k;
      if (FRAME && X0 + lx >= nx) break;  // uniform per warp: rows past the grid's last
      const float2 txzl = lds2(&TXZ[r][cc - 2]), txzr = lds2(&TXZ[r][cc + 2]);
      const float2 tzzl = lds2(&TZZ[r][cc - 2]), tzz0 = lds2(&TZZ[r][cc]),
                   tzzr = lds2(&TZZ[r][cc + 2]);
      const float ax0 = (c1x * (a0.x - am1.x) + c2x * (am2.x - ap1.x)) +
                        (c1z * (b0.x - txzl.y) + c2z * (txzl.x - b0.y));
      const float ax1 = (c1x * (a0.y - am1.y) + c2x * (am2.y - ap1.y)) +
                        (c1z * (b0.y - b0.x) + c2z * (txzl.y - txzr.x));
      const float az0 = (c1x * (bp1.x - b0.x) + c2x * (bm1.x - bp2.x)) +
                        (c1z * (tzz0.y - tzz0.x) + c2z * (tzzl.y - tzzr.x));
      const float az1 = (c1x * (bp1.y - b0.y) + c2x * (bm1.y - bp2.y)) +
                        (c1z * (tzzr.x - tzz0.y) + c2z * (tzz0.x - tzzr.y));
      float2 vx = lds2(&VX[lx + 4][cc]), vz = lds2(&VZ[lx + 4][cc]);
      const float bdt0 = bb[2 * k] * dtv, bdt1 = bb[2 * k + 1] * dtv;
      const float nvx0 = vx.x + bdt0 * ax0, nvx1 = vx.y + bdt1 * ax1;
      const float nvz0 = vz.x + bdt0 * az0, nvz1 = vz.y + bdt1 * az1;
      if (FRAME) {
        const int gx = X0 + lx;
        const bool xi = gx >= 2 && gx < nx - 2;
        const float tr = axis_taper(d, gx, nx);
        const float t0 = fminf(tz0, tr), t1 = fminf(tz1, tr);
        const bool u0 = xi && zi0, u1 = xi && zi1;
        vx.x = u0 ? t0 * nvx0 : vx.x;
        vz.x = u0 ? t0 * nvz0 : vz.x;
        vx.y = u1 ? t1 * nvx1 : vx.y;
        vz.y = u1 ? t1 * nvz1 : vz.y;
      } else {
        vx = make_float2(nvx0, nvx1);
        vz = make_float2(nvz0, nvz1);
      }
      sts2(out.vx + gq, vx);
      sts2(out.vz + gq, vz);
      gq += ps;
      if (k + 1 < KV) {
        am2 = am1;
        am1 = a0;
        a0 = ap1;
        ap1 = lds2(&TXX[r + 2][cc]);
        bm1 = b0;
        b0 = bp1;
        bp1 = bp2;
        bp2 = lds2(&TXZ[r + 3][cc]);
      }
    }
  }
}

// One tile's time step. `maps` are the tensor maps of this step's input set;
// the kernels below pass them either as a kernel parameter (single model:
// the copies can be issued without waiting for any load) or from the
// descriptor table (batch).
// TAPERED: taper tiles take the interior path with the taper factor. On for
// the 128-thread shapes (small and mid-size grids, where the absorbing frame
// holds many tiles: +3.5 % on the batched and surrogate workloads); off for
// 32 x 60, whose 2100 x 900 persistent step it slowed by 1.5 %. A shape
// uses the same paths in every kernel, so per-step and persistent launches
// give the same bits.
template <class S, int CFG, bool ADJ, bool TAPERED = (S::NT == 128), class Mid = NoHook>
__device__ __forceinline__ bool step_body(const SimDesc &d, const Maps &maps, int X0, int Z0,
                                          bool first, int tile, int it, int parity, int store,
                                          int *err, uint32_t phase, bool init_bar,
                                          bool sync_copy = true, const Mid &mid = Mid()) {
  constexpr int TX = S::TX, TZ = S::TZ, W = S::W, VR = S::VR, SR = S::SR, G = S::G;
  extern __shared__ unsigned char smem_raw[];
  unsigned char *base = reinterpret_cast<unsigned char *>(
      (reinterpret_cast<uintptr_t>(smem_raw) + 127) & ~static_cast<uintptr_t>(127));
  float(*sv)[VR][W] = reinterpret_cast<float(*)[VR][W]>(base);  // vx, vz (VPITCH each)
  float(*sv1)[W] = reinterpret_cast<float(*)[W]>(base + S::VPITCH);
  auto stile = [&](int k) {  // txx tzz txz lm mu
    return reinterpret_cast<float(*)[W]>(base + 2 * S::VPITCH + k * S::SPITCH);
  };
  float(*const sxx_)[W] = stile(0);
  float(*const szz_)[W] = stile(1);
  float(*const sxz_)[W] = stile(2);
  float(*const slm)[W] = stile(3);
  float(*const smu)[W] = stile(4);
  uint64_t *bar = reinterpret_cast<uint64_t *>(base + S::TILE_BYTES);

  const int nx = d.nx, nz = d.nz, ps = d.pitch;
  const fast::Fields out = d.set[parity ^ 1];
  const float c1 = 9.0f / 8.0f, c2 = 1.0f / 24.0f;

  if (threadIdx.x == 0 && init_bar) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(1)
                 : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  // Snapshot step: forward stores the pre-step state, adjoint correlates
  // with it (both at this shot's snapshot it / si).
  const bool snap_io = (it % d.si) == 0 && d.accu[0] != nullptr && (ADJ || store);
  const size_t soff = (size_t)(it / d.si) * nx * nz;
  const bool inner = interior_tile<S>(d, X0, Z0, snap_io);
  // The 60-column shapes take the vectorised path on interior and frame
  // tiles; the 28-column shapes keep the one-column paths (interior and
  // taper).
  constexpr bool V2 = S::TZ == 60;
  const bool frame = V2 && !inner && frame_tile<S>(d, X0, Z0, snap_io);
  const bool tapered = TAPERED && !inner && taper_tile<S>(d, X0, Z0, snap_io);
  // One-column shapes: the other tiles without snapshot I/O or injection
  // take the register-window path with masks (frame tiles).
  const bool frame1 = TAPERED && !V2 && !inner && !tapered && !snap_io &&
                      !injection_tile<S>(d, X0, Z0);

  // This thread's buoyancy values for phase C (the medium does not change
  // between steps, so they load before the previous step has finished).
  // Interior tiles give each row group consecutive rows, the others every
  // G-th row.
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, h = w % S::H, q = w / S::H;
  constexpr int KC = TX / G;  // own rows per thread
  const int lzc = h * 32 + lane;  // own column of this thread (valid if < TZ)
  const int gzc = Z0 + lzc;
  const bool col_ok = lzc < TZ && gzc < nz;
  float bb[KC];
  if (V2 && (inner || frame)) {
    // Two columns per lane (lanes 0-29), rows X0 + KV w + k: own points (the
    // columns inside the grid; rows past its last row read nothing).
    constexpr int KV = TX / S::WARPS;
    static_assert(!V2 || KC == 2 * KV, "KV rows of two columns per thread");
#pragma unroll
    for (int k = 0; k < KV; ++k) {
      float2 v = make_float2(0.f, 0.f);
      if (lane < TZ / 2 && X0 + KV * w + k < nx)
        v = __ldg(reinterpret_cast<const float2 *>(d.b + (X0 + KV * w + k) * ps + Z0 + 2 * lane));
      bb[2 * k] = v.x;
      bb[2 * k + 1] = v.y;
    }
  } else {
#pragma unroll
    for (int k = 0; k < KC; ++k) {
      const int gx = (inner || tapered || frame1) ? X0 + q * KC + k : X0 + q + G * k;
      bb[k] = (col_ok && gx < nx) ? __ldg(d.b + gx * ps + gzc) : 0.f;
    }
  }
  griddep_wait();
  // (sync_copy false: the caller has just passed a barrier that follows
  // every thread's last access of the tile buffers, and the mbarrier is
  // initialised.)
  if (sync_copy) __syncthreads();
  if (threadIdx.x == 0) {
    // Order this CTA's earlier generic accesses of the tile buffers before
    // the copies overwrite them.
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)),
                 "r"(S::TX_BYTES)
                 : "memory");
    tma_load_2d(&sv[0][0][0], &maps.vx, Z0 - 4, X0 - 4, bar);
    tma_load_2d(&sv1[0][0], &maps.vz, Z0 - 4, X0 - 4, bar);
    tma_load_2d(&sxx_[0][0], &maps.txx, Z0 - 4, X0 - 2, bar);
    tma_load_2d(&szz_[0][0], &maps.tzz, Z0 - 4, X0 - 2, bar);
    tma_load_2d(&sxz_[0][0], &maps.txz, Z0 - 4, X0 - 2, bar);
    tma_load_2d(&slm[0][0], &maps.lm, Z0 - 4, X0 - 2, bar);
    tma_load_2d(&smu[0][0], &maps.mu, Z0 - 4, X0 - 2, bar);
  }
  griddep_launch_dependents();

  // While the copies fly: receivers (pre-step velocities, by the first tile
  // of each simulation).
  if (!ADJ && first && d.nr) {
    const float *in_vx = d.set[parity].vx, *in_vz = d.set[parity].vz;
    for (int r = threadIdx.x; r < d.nr; r += S::NT) {
      const int c = d.rec_cell[r];
      d.rec_vx[(size_t)r * d.nt + it] = in_vx[c];
      d.rec_vz[(size_t)r * d.nt + it] = in_vz[c];
    }
  }

  // Bounded wait (about a second at most); the CTA agrees on the outcome so
  // that it leaves together, after its copies have landed.
  const bool landed = mbar_wait(bar, phase, 1u << 20);
  if (__syncthreads_or(!landed)) {
    if (threadIdx.x == 0) {
      atomicOr(err, 1);
      mbar_wait(bar, phase, 1u << 20);
    }
    return false;
  }
  // Persistent step: the tile records its own receivers (pre-step
  // velocities) from the copied tile.
  if (!ADJ && tile >= 0 && d.rec_start) {
    const int r1 = d.rec_start[tile + 1];
    for (int i = d.rec_start[tile] + threadIdx.x; i < r1; i += S::NT) {
      const int r = d.rec_list[i];
      const int c = d.rec_cell[r];
      const int ix = c / ps, iz = c - ix * ps;
      d.rec_vx[(size_t)r * d.nt + it] = sv[0][ix - X0 + 4][iz - Z0 + 4];
      d.rec_vz[(size_t)r * d.nt + it] = sv1[ix - X0 + 4][iz - Z0 + 4];
    }
  }

  const float dtv = ADJ ? -d.dt : d.dt;
  const float idx = d.idx, idz = d.idz;
  const float(*VX)[W] = sv[0];
  const float(*VZ)[W] = sv1;

  if constexpr (V2) {
    if (inner) {
      tile_phases_v2<S, ADJ, false>(d, out, X0, Z0, VX, VZ, sxx_, szz_, sxz_, slm, smu, bb, mid);
      return true;
    }
    if (frame) {
      tile_phases_v2<S, ADJ, true>(d, out, X0, Z0, VX, VZ, sxx_, szz_, sxz_, slm, smu, bb, mid);
      return true;
    }
  } else {
    if (inner) {
      tile_phases<S, ADJ, false>(d, out, X0, Z0, VX, VZ, sxx_, szz_, sxz_, slm, smu, bb, mid);
      return true;
    }
  }
  if (TAPERED && tapered) {
    tile_phases<S, ADJ, true>(d, out, X0, Z0, VX, VZ, sxx_, szz_, sxz_, slm, smu, bb, mid);
    return true;
  }
  if (TAPERED && frame1) {
    tile_phases<S, ADJ, true, true>(d, out, X0, Z0, VX, VZ, sxx_, szz_, sxz_, slm, smu, bb, mid);
    return true;
  }

  const int np = d.np;
  // Phase B: new stresses over rows X0-2 .. X0+TX+2 and box columns
  // 2 .. TZ+6 (z = Z0-2 .. Z0+TZ+2), in place.
  {
    const int c = 2 + h * 32 + lane;  // box column
    const int gz = Z0 - 4 + c;
    const bool z_in = gz >= 0 && gz < nz;
    const bool z_int = gz >= 2 && gz < nz - 2;
    const bool z_own = c >= 4 && c < TZ + 4;
    const bool z_free = gz >= d.fz0 && gz < d.fz1;
    const int tz = min(gz + 1, nz - gz);
#pragma unroll 3
    for (int k = 0; k < SR / G; ++k) {
      const int r = q + G * k;  // box row
      const int gx = X0 - 2 + r;
      if (!z_in || gx < 0 || gx >= nx) continue;
      const int g = gx * nz + gz;   // unpadded (snapshots, kernels)
      const int gp = gx * ps + gz;  // padded (wave fields)
      const int vr = r + 2;         // same point in the velocity box
      float sxx = sxx_[r][c], szz = szz_[r][c], sxz = sxz_[r][c];
      const bool own = z_own && r >= 2 && r < TX + 2;
      if (!ADJ && own && snap_io) {
        d.accu[0][soff + g] = VX[vr][c];
        d.accu[1][soff + g] = VZ[vr][c];
        d.accu[2][soff + g] = sxx;
        d.accu[3][soff + g] = szz;
        d.accu[4][soff + g] = sxz;
      }
      const float lm = slm[r][c], mu = smu[r][c];
      if (ADJ && own && snap_io && z_free && gx >= d.fx0 && gx < d.fx1) {
        const float *asnap[5] = {d.accu[0] + soff, d.accu[1] + soff, d.accu[2] + soff,
                                 d.accu[3] + soff, d.accu[4] + soff};
        correlate(d, asnap, g, lm, mu, VX[vr][c], VZ[vr][c], sxx, szz, sxz);
      }
      if (z_int && gx >= 2 && gx < nx - 2) {
        const float la = lm - 2.0f * mu;
        const float dvx = c1 * (VX[vr + 1][c] - VX[vr][c]) + c2 * (VX[vr - 1][c] - VX[vr + 2][c]);
        const float dvz = c1 * (VZ[vr][c] - VZ[vr][c - 1]) + c2 * (VZ[vr][c - 2] - VZ[vr][c + 1]);
        const float gxz = (c1 * (VX[vr][c + 1] - VX[vr][c]) +
                           c2 * (VX[vr][c - 1] - VX[vr][c + 2])) * idz +
                          (c1 * (VZ[vr][c] - VZ[vr - 1][c]) +
                           c2 * (VZ[vr - 2][c] - VZ[vr + 1][c])) * idx;
        const float ex = dvx * idx, ez = dvz * idz;
        // Points at least np frames deep have taper exp(0) = 1 exactly.
        const int cnt = min(tz, min(gx + 1, nx - gx));
        const float tp = cnt < np ? __ldg(d.taper_tab + cnt) : 1.0f;
        sxx = tp * (sxx + dtv * (lm * ex + la * ez));
        szz = tp * (szz + dtv * (la * ex + lm * ez));
        sxz = tp * (sxz + dtv * mu * gxz);
        sxx_[r][c] = sxx;
        szz_[r][c] = szz;
        sxz_[r][c] = sxz;
      }
      if (own) {
        out.txx[gp] = sxx;
        out.tzz[gp] = szz;
        out.txz[gp] = sxz;
      }
    }
  }
  __syncthreads();
  mid();

  // Phase C: new velocities of the tile's own points.
  if (col_ok) {
    const float(*TXX)[W] = sxx_;
    const float(*TZZ)[W] = szz_;
    const float(*TXZ)[W] = sxz_;
    const InjPlan &p = d.plan;
    const int c = lzc + 4;  // box column of this thread's points
    const bool z_int = gzc >= 2 && gzc < nz - 2;
    const int tz = min(gzc + 1, nz - gzc);
    const bool z_box = p.n && gzc >= p.z0 && gzc < p.z0 + p.h;
#pragma unroll
    for (int k = 0; k < KC; ++k) {
      const int lx = q + G * k;
      const int gx = X0 + lx;
      if (gx >= nx) continue;
      const int g = gx * nz + gzc;   // unpadded (injection cells)
      const int gp = gx * ps + gzc;  // padded
      const int r = lx + 2;          // stress box row
      float vx = VX[lx + 4][c], vz = VZ[lx + 4][c];
      const float b = bb[k];
      if (z_int && gx >= 2 && gx < nx - 2) {
        const float ax = (c1 * (TXX[r][c] - TXX[r - 1][c]) + c2 * (TXX[r - 2][c] - TXX[r + 1][c])) * idx +
                         (c1 * (TXZ[r][c] - TXZ[r][c - 1]) + c2 * (TXZ[r][c - 2] - TXZ[r][c + 1])) * idz;
        const float az = (c1 * (TXZ[r + 1][c] - TXZ[r][c]) + c2 * (TXZ[r - 1][c] - TXZ[r + 2][c])) * idx +
                         (c1 * (TZZ[r][c + 1] - TZZ[r][c]) + c2 * (TZZ[r][c - 1] - TZZ[r][c + 2])) * idz;
        const int cnt = min(tz, min(gx + 1, nx - gx));
        const float tp = cnt < np ? __ldg(d.taper_tab + cnt) : 1.0f;
        const float bdt = b * dtv;
        vx = tp * (vx + bdt * ax);
        vz = tp * (vz + bdt * az);
      }
      if (z_box && gx >= p.x0 && gx < p.x0 + p.w) inject(d, it, g, gx, gzc, b, vx, vz);
      out.vx[gp] = vx;
      out.vz[gp] = vz;
    }
  }
  return true;
}

// Single simulation: tensor maps as a parameter, tiles from blockIdx
// (row-major over tiles_z tile columns).
template <class S, int CFG, bool ADJ>
__global__ void __launch_bounds__(S::NT, S::MINB)
    fused_step_tma(const __grid_constant__ SimDesc d, int tiles_z, int it, int parity, int store,
                   int *err) {
  const int bx = blockIdx.x, tx = bx / tiles_z, tz = bx - tx * tiles_z;
  step_body<S, CFG, ADJ>(d, d.maps[parity], tx * S::TX, tz * S::TZ, bx == 0, -1, it, parity,
                         store, err, 0u, true);
}

// Many simulations: tile table entries (sim, x0, z0, first) per CTA. With
// `active` non-null, the CTAs of simulations whose flag is 0 return at once.
template <class S, int CFG, bool ADJ>
__global__ void __launch_bounds__(S::NT, S::MINB)
    fused_step_tma_batch(const SimDesc *__restrict__ sims, const int4 *__restrict__ tiles,
                         const int *__restrict__ active, int it, int parity, int store, int *err) {
  const int4 t = tiles[blockIdx.x];
  if (active && !active[t.x]) return;
  const SimDesc &d = sims[t.x];
  step_body<S, CFG, ADJ>(d, d.maps[parity], t.y, t.z, t.w != 0, -1, it, parity, store, err, 0u,
                         true);
}

// Bounded wait until the counter at p reaches v (acquire): true when it did.
// After 64 plain polls each round sleeps about 100 ns; 2^22 rounds bound
// the wait to a few seconds at most.
__device__ __forceinline__ bool wait_at_least(const unsigned *p, unsigned v) {
  for (uint32_t i = 0; i < (1u << 22); ++i) {
    unsigned x;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(x) : "l"(p) : "memory");
    if (x >= v) return true;
    if (i >= 64) __nanosleep(100);  // poll first: most waits are short
  }
  return false;
}

// All time steps of one simulation in one launch. sched[0] hands out items
// w = step * n_tiles + tile in increasing order; sched[1 + t] counts the
// steps tile t has finished. An item starts once the tile and its eight
// neighbours have finished the previous step: that is everything the step
// reads (halos are at most 4 points, less than a tile), and it also
// guarantees that no neighbour still reads the buffer the step overwrites.
// The earliest unfinished item always has its inputs ready, so the
// schedule cannot deadlock; each wait is bounded nonetheless, and a CTA
// that gives up raises *err and stops (its dependents then time out too).
//
// Thread 0 draws the CTA's next item between phases B and C of the current
// one: the atomic's latency hides behind phase C, and a CTA holds a second
// item only for that last part of an item. Drawn earlier, the CTAs held
// about one step's worth of items between them (456 CTAs, 990 tiles), so
// an item often reached its neighbours' previous step before they had
// finished it.
// Publication: after the item's closing barrier the last thread of the CTA
// (idle in phase C) issues one st.release.gpu. Release is cumulative, so it
// orders every store of the CTA that precedes the barrier, and the waiting
// side's ld.acquire.gpu sees them all; its wait for the item's stores to
// drain overlaps the next item's polls and copies.
template <class S, int CFG, bool ADJ>
__global__ void __launch_bounds__(S::NT, S::MINB)
    fused_steps_tma(const __grid_constant__ SimDesc d, int tiles_x, int tiles_z, int it0,
                    int n_steps, int parity0, int store, int *err, unsigned *sched) {
  __shared__ int s_item;
  const int n_tiles = tiles_x * tiles_z;
  const long long total = (long long)n_steps * n_tiles;
  constexpr int PUB = S::NT - 1;
  uint32_t phase = 0;
  bool init = true;
  unsigned next = 0;
  if (threadIdx.x == 0) s_item = (int)atomicAdd(sched, 1u);
  __syncthreads();
  for (;;) {
    const long long w = s_item;
    if (w >= total) return;
    const int j = (int)(w / n_tiles), tile = (int)(w - (long long)j * n_tiles);
    const int tx = tile / tiles_z, tz = tile - tx * tiles_z;
    bool ok = true;
    if (j > 0 && threadIdx.x >= 32 && threadIdx.x < 41) {
      const int k = (int)threadIdx.x - 32;
      const int a = tx + k / 3 - 1, b = tz + k % 3 - 1;
      if (a >= 0 && a < tiles_x && b >= 0 && b < tiles_z)
        ok = wait_at_least(sched + 1 + a * tiles_z + b, (unsigned)j);
    }
    if (!__syncthreads_and(ok)) {
      if (threadIdx.x == 0) atomicOr(err, 2);
      return;
    }
    if (j > 0 && threadIdx.x == 0) asm volatile("fence.proxy.async.global;" ::: "memory");
    const int it = ADJ ? it0 - j : it0 + j;
    const int parity = parity0 ^ (j & 1);
    const auto draw = [&]() {
      if (threadIdx.x == 0) next = atomicAdd(sched, 1u);
    };
    if (!step_body<S, CFG, ADJ, (S::NT == 128)>(d, d.maps[parity], tx * S::TX, tz * S::TZ, false,
                                                 tile, it, parity, store, err, phase, init,
                                                 init, draw))
      return;
    phase ^= 1u;
    init = false;
    if (threadIdx.x == 0) s_item = (int)next;
    __syncthreads();
    if (threadIdx.x == PUB)
      asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(sched + 1 + tile),
                   "r"((unsigned)(j + 1))
                   : "memory");
  }
}

// The persistent step over a batch's tile table: items w = step * n_tiles +
// k for table entries k (simulation, x0, z0, first); neighbours are the
// tiles of the same simulation around it. Same schedule, waits and
// publication as fused_steps_tma; inactive simulations' items are skipped
// (their neighbours are inactive too).
template <class S, int CFG>
__global__ void __launch_bounds__(S::NT, S::MINB)
    fused_steps_tma_batch(const SimDesc *__restrict__ sims, const int4 *__restrict__ tiles,
                          const int *__restrict__ active, int n_tiles, int n_steps, int store,
                          int *err, unsigned *sched) {
  __shared__ int s_item;
  const long long total = (long long)n_steps * n_tiles;
  uint32_t phase = 0;
  bool init = true;
  // As fused_steps_tma: thread 0 publishes the finished item while warp 1
  // polls the new item's neighbours.
  unsigned next = 0;
  int pub = -1;
  unsigned pub_count = 0;
  if (threadIdx.x == 0) {
    s_item = (int)atomicAdd(sched, 1u);
    next = atomicAdd(sched, 1u);
  }
  __syncthreads();
  for (;;) {
    const long long w = s_item;
    if (w >= total) {
      if (threadIdx.x == 0 && pub >= 0)
        asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(sched + 1 + pub),
                     "r"(pub_count)
                     : "memory");
      return;
    }
    const int j = (int)(w / n_tiles), k = (int)(w - (long long)j * n_tiles);
    const int4 t = tiles[k];
    const bool skip = active && !active[t.x];  // uniform: t is the CTA's
    const SimDesc &d = sims[t.x];
    const int tx = t.y / S::TX, tz = t.z / S::TZ;
    bool ok = true;
    if (!skip && j > 0 && threadIdx.x >= 32 && threadIdx.x < 41) {
      const int q = (int)threadIdx.x - 32;
      const int a = tx + q / 3 - 1, b = tz + q % 3 - 1;
      if (a >= 0 && a < d.tiles_x && b >= 0 && b < d.tiles_z)
        ok = wait_at_least(sched + 1 + d.tile_base + a * d.tiles_z + b, (unsigned)j);
    }
    if (threadIdx.x == 0 && pub >= 0) {
      asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(sched + 1 + pub),
                   "r"(pub_count)
                   : "memory");
      pub = -1;
    }
    if (!__syncthreads_and(ok)) {
      if (threadIdx.x == 0) atomicOr(err, 2);
      return;
    }
    if (!skip) {
      if (j > 0 && threadIdx.x == 0) asm volatile("fence.proxy.async.global;" ::: "memory");
      const int parity = j & 1;
      if (!step_body<S, CFG, false>(d, d.maps[parity], t.y, t.z, false, tx * d.tiles_z + tz, j,
                                    parity, store, err, phase, init, init))
        return;
      phase ^= 1u;
      init = false;
      if (threadIdx.x == 0) {
        pub = k;
        pub_count = (unsigned)(j + 1);
      }
    }
    if (threadIdx.x == 0) {
      s_item = (int)next;
      next = atomicAdd(sched, 1u);
    }
    __syncthreads();  // the item's stores are issued; s_item is the next item
  }
}

// The shared-memory opt-in is a per-device attribute: set it once per device.
template <class K>
cudaError_t configure(K kernel, int smem, unsigned long long &configured) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  const unsigned long long bit = 1ull << (dev & 63);
  if (!(configured & bit)) {
    e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    if (e != cudaSuccess) return e;
    configured |= bit;
  }
  return cudaSuccess;
}

template <class S, int CFG, bool ADJ>
cudaError_t launch(const SimDesc *sims, const int4 *tiles, int n_tiles, const int *active, int it,
                   int parity, int store, int *err, cudaStream_t s) {
  static unsigned long long configured = 0;
  cudaError_t e = configure(fused_step_tma_batch<S, CFG, ADJ>, S::SMEM, configured);
  if (e != cudaSuccess) return e;
  if (n_tiles <= 0) return cudaSuccess;
  // Programmatic stream serialisation, as for the single-model step: the
  // CTAs of this step may become resident while the previous step's last
  // wave drains; they wait in griddep_wait before touching any wave field.
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  cudaLaunchConfig_t lc = {};
  lc.gridDim = dim3(n_tiles);
  lc.blockDim = dim3(S::NT);
  lc.dynamicSmemBytes = S::SMEM;
  lc.stream = s;
  lc.attrs = attr;
  lc.numAttrs = 1;
  return cudaLaunchKernelEx(&lc, fused_step_tma_batch<S, CFG, ADJ>, sims, tiles, active, it,
                            parity, store, err);
}

template <class S, int CFG, bool ADJ>
cudaError_t launch_persistent(const SimDesc &d, int it0, int n_steps, int parity0, int store,
                              int *err, unsigned *sched, cudaStream_t s) {
  static unsigned long long configured = 0;
  cudaError_t e = configure(fused_steps_tma<S, CFG, ADJ>, S::SMEM, configured);
  if (e != cudaSuccess) return e;
  if (n_steps <= 0) return cudaSuccess;
  const int tiles_x = (d.nx + S::TX - 1) / S::TX, tiles_z = (d.nz + S::TZ - 1) / S::TZ;
  int dev = 0, sms = 0, per_sm = 0;
  if ((e = cudaGetDevice(&dev)) != cudaSuccess) return e;
  if ((e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev)) != cudaSuccess)
    return e;
  if ((e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fused_steps_tma<S, CFG, ADJ>,
                                                         S::NT, S::SMEM)) != cudaSuccess)
    return e;
  const long long items = (long long)n_steps * tiles_x * tiles_z;
  // At most the resident CTAs, and at most two steps' worth of tiles: more
  // CTAs would only hold items further ahead and poll for them.
  const long long slots = (long long)std::max(per_sm, 1) * sms;
  const int grid = (int)std::min(std::min<long long>(items, slots), 2LL * tiles_x * tiles_z);
  // Item numbers are 31-bit: a CTA draws two numbers up front and one per
  // item, so the counter reaches at most items + 2 * grid - 1.
  if (items + 2LL * grid >= 0x7fffffffLL) return cudaErrorInvalidValue;
  // Cooperative launch: every CTA is resident at once, as CTAs that wait on
  // one another require.
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeCooperative;
  attr[0].val.cooperative = 1;
  cudaLaunchConfig_t lc = {};
  lc.gridDim = dim3(grid);
  lc.blockDim = dim3(S::NT);
  lc.dynamicSmemBytes = S::SMEM;
  lc.stream = s;
  lc.attrs = attr;
  lc.numAttrs = 1;
  return cudaLaunchKernelEx(&lc, fused_steps_tma<S, CFG, ADJ>, d, tiles_x, tiles_z, it0, n_steps,
                            parity0, store, err, sched);
}

template <class S, int CFG, bool ADJ>
cudaError_t launch_single(const SimDesc &d, int it, int parity, int store, int *err,
                          cudaStream_t s) {
  static unsigned long long configured = 0;
  cudaError_t e = configure(fused_step_tma<S, CFG, ADJ>, S::SMEM, configured);
  if (e != cudaSuccess) return e;
  const int tiles_x = (d.nx + S::TX - 1) / S::TX, tiles_z = (d.nz + S::TZ - 1) / S::TZ;
  // Programmatic stream serialisation: the CTAs of this step may become
  // resident while the previous step drains; they wait in griddep_wait
  // before touching any wave field.
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  cudaLaunchConfig_t lc = {};
  lc.gridDim = dim3(tiles_x * tiles_z);
  lc.blockDim = dim3(S::NT);
  lc.dynamicSmemBytes = S::SMEM;
  lc.stream = s;
  lc.attrs = attr;
  lc.numAttrs = 1;
  return cudaLaunchKernelEx(&lc, fused_step_tma<S, CFG, ADJ>, d, tiles_z, it, parity, store, err);
}

using EncodeTiled = CUresult (*)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *,
                                 const cuuint64_t *, const cuuint64_t *, const cuuint32_t *,
                                 const cuuint32_t *, CUtensorMapInterleave, CUtensorMapSwizzle,
                                 CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

EncodeTiled encoder() {
  static EncodeTiled fn = nullptr;
  if (!fn) {
    void *p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault,
                                         &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<EncodeTiled>(p);
  }
  return fn;
}

bool encode(CUtensorMap *m, const float *ptr, int nx, int nz, int pitch, int width, int rows) {
  EncodeTiled fn = encoder();
  if (!fn) return false;
  const cuuint64_t dims[2] = {(cuuint64_t)nz, (cuuint64_t)nx};
  const cuuint64_t strides[1] = {(cuuint64_t)pitch * sizeof(float)};
  const cuuint32_t box[2] = {(cuuint32_t)width, (cuuint32_t)rows};
  const cuuint32_t elem[2] = {1, 1};
  return fn(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, const_cast<float *>(ptr), dims, strides, box,
            elem, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
            CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) ==
         CUDA_SUCCESS;
}

template <class S>
bool encode_set(Maps &m, const fast::Fields &f, const float *lm, const float *mu, int nx, int nz,
                int pitch) {
  return encode(&m.vx, f.vx, nx, nz, pitch, S::W, S::VR) &&
         encode(&m.vz, f.vz, nx, nz, pitch, S::W, S::VR) &&
         encode(&m.txx, f.txx, nx, nz, pitch, S::W, S::SR) &&
         encode(&m.tzz, f.tzz, nx, nz, pitch, S::W, S::SR) &&
         encode(&m.txz, f.txz, nx, nz, pitch, S::W, S::SR) &&
         encode(&m.lm, lm, nx, nz, pitch, S::W, S::SR) &&
         encode(&m.mu, mu, nx, nz, pitch, S::W, S::SR);
}

}  // namespace

bool encode_2d(CUtensorMap *m, const float *ptr, int nx, int nz, int pitch, int width, int rows) {
  return encode(m, ptr, nx, nz, pitch, width, rows);
}

bool encode_planes(CUtensorMap *m, const float *base, int planes, size_t plane_bytes, int nx,
                   int nz, int pitch, int width, int rows) {
  EncodeTiled fn = encoder();
  if (!fn || plane_bytes % 16 != 0) return false;
  const cuuint64_t dims[3] = {(cuuint64_t)nz, (cuuint64_t)nx, (cuuint64_t)planes};
  const cuuint64_t strides[2] = {(cuuint64_t)pitch * sizeof(float), (cuuint64_t)plane_bytes};
  const cuuint32_t box[3] = {(cuuint32_t)width, (cuuint32_t)rows, 1};
  const cuuint32_t elem[3] = {1, 1, 1};
  return fn(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, const_cast<float *>(base), dims, strides, box,
            elem, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
            CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) ==
         CUDA_SUCCESS;
}

void tile_dims(int cfg, int *tx, int *tz) {
  with_shape(cfg, [&](auto t) {
    using S = typename decltype(t)::S;
    *tx = S::TX;
    *tz = S::TZ;
    return 0;
  });
}

bool supported(int nx, int nz, int pitch) {
  return pitch % 4 == 0 && pitch >= nz && nx > 0 && nz > 0 && encoder() != nullptr;
}

bool make_maps(SimDesc &d, const float *mu, int cfg) {
  for (int p = 0; p < 2; ++p) {
    const bool ok = with_shape(cfg, [&](auto t) {
      using S = typename decltype(t)::S;
      return encode_set<S>(d.maps[p], d.set[p], d.lm, mu, d.nx, d.nz, d.pitch);
    });
    if (!ok) return false;
  }
  return true;
}

bool encode_input_maps(Maps &m, const fast::Fields &in, const float *lm, const float *mu, int nx,
                       int nz, int pitch, int cfg) {
  return with_shape(cfg, [&](auto t) {
    using S = typename decltype(t)::S;
    return encode_set<S>(m, in, lm, mu, nx, nz, pitch);
  });
}

void append_tiles(int cfg, int sim, int nx, int nz, std::vector<int4> &tiles) {
  int tx, tz;
  tile_dims(cfg, &tx, &tz);
  bool first = true;
  for (int x0 = 0; x0 < nx; x0 += tx)
    for (int z0 = 0; z0 < nz; z0 += tz) {
      tiles.push_back(make_int4(sim, x0, z0, first ? 1 : 0));
      first = false;
    }
}

cudaError_t step_single(const SimDesc &d, int cfg, bool adjoint, int it, int parity, bool store,
                        int *err, cudaStream_t s) {
  const int st = store ? 1 : 0;
  return with_shape(cfg, [&](auto t) {
    using S = typename decltype(t)::S;
    constexpr int CFG = decltype(t)::CFG;
    return adjoint ? launch_single<S, CFG, true>(d, it, parity, st, err, s)
                   : launch_single<S, CFG, false>(d, it, parity, st, err, s);
  });
}

int tile_count(int cfg, int nx, int nz) {
  int tx, tz;
  tile_dims(cfg, &tx, &tz);
  return ((nx + tx - 1) / tx) * ((nz + tz - 1) / tz);
}

int tile_of(int cfg, int nz, int ix, int iz) {
  int tx, tz;
  tile_dims(cfg, &tx, &tz);
  return (ix / tx) * ((nz + tz - 1) / tz) + iz / tz;
}

size_t sched_words(int cfg, int nx, int nz) { return 1 + (size_t)tile_count(cfg, nx, nz); }

namespace {
template <class S, int CFG, bool ADJ>
int resident() {
  static unsigned long long configured = 0;
  if (configure(fused_steps_tma<S, CFG, ADJ>, S::SMEM, configured) != cudaSuccess) return 0;
  int dev = 0, sms = 0, per_sm = 0;
  if (cudaGetDevice(&dev) != cudaSuccess ||
      cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess ||
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fused_steps_tma<S, CFG, ADJ>, S::NT,
                                                    S::SMEM) != cudaSuccess)
    return 0;
  return per_sm * sms;
}
}  // namespace

template <class S, int CFG>
cudaError_t launch_persistent_batch(const SimDesc *sims, const int4 *tiles, int n_tiles,
                                    const int *active, int n_steps, int store, int *err,
                                    unsigned *sched, cudaStream_t s) {
  static unsigned long long configured = 0;
  cudaError_t e = configure(fused_steps_tma_batch<S, CFG>, S::SMEM, configured);
  if (e != cudaSuccess) return e;
  if (n_steps <= 0 || n_tiles <= 0) return cudaSuccess;
  int dev = 0, sms = 0, per_sm = 0;
  if ((e = cudaGetDevice(&dev)) != cudaSuccess) return e;
  if ((e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev)) != cudaSuccess)
    return e;
  if ((e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fused_steps_tma_batch<S, CFG>,
                                                         S::NT, S::SMEM)) != cudaSuccess)
    return e;
  const long long items = (long long)n_steps * n_tiles;
  const long long slots = (long long)std::max(per_sm, 1) * sms;
  const int grid = (int)std::min(std::min<long long>(items, slots), 2LL * n_tiles);
  if (items + 2LL * grid >= 0x7fffffffLL) return cudaErrorInvalidValue;  // 31-bit items
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeCooperative;
  attr[0].val.cooperative = 1;
  cudaLaunchConfig_t lc = {};
  lc.gridDim = dim3(grid);
  lc.blockDim = dim3(S::NT);
  lc.dynamicSmemBytes = S::SMEM;
  lc.stream = s;
  lc.attrs = attr;
  lc.numAttrs = 1;
  return cudaLaunchKernelEx(&lc, fused_steps_tma_batch<S, CFG>, sims, tiles, active, n_tiles,
                            n_steps, store, err, sched);
}

size_t sched_words_batch(int n_tiles) { return 1 + (size_t)std::max(n_tiles, 0); }

cudaError_t steps_persistent_batch(const SimDesc *sims, const int4 *tiles, int n_tiles,
                                   const int *active, int cfg, int n_steps, bool store, int *err,
                                   unsigned *sched, cudaStream_t s) {
  const int st = store ? 1 : 0;
  return with_shape(cfg, [&](auto t) {
    using S = typename decltype(t)::S;
    constexpr int CFG = decltype(t)::CFG;
    return launch_persistent_batch<S, CFG>(sims, tiles, n_tiles, active, n_steps, st, err, sched,
                                           s);
  });
}

int resident_ctas(int cfg, bool adjoint) {
  return with_shape(cfg, [&](auto t) {
    using S = typename decltype(t)::S;
    constexpr int CFG = decltype(t)::CFG;
    return adjoint ? resident<S, CFG, true>() : resident<S, CFG, false>();
  });
}

cudaError_t steps_persistent(const SimDesc &d, int cfg, bool adjoint, int it0, int n_steps,
                             int parity0, bool store, int *err, unsigned *sched, cudaStream_t s) {
  const int st = store ? 1 : 0;
  return with_shape(cfg, [&](auto t) {
    using S = typename decltype(t)::S;
    constexpr int CFG = decltype(t)::CFG;
    return adjoint ? launch_persistent<S, CFG, true>(d, it0, n_steps, parity0, st, err, sched, s)
                   : launch_persistent<S, CFG, false>(d, it0, n_steps, parity0, st, err, sched, s);
  });
}

cudaError_t step(const SimDesc *sims, const int4 *tiles, int n_tiles, const int *active, int cfg,
                 bool adjoint, int it, int parity, bool store, int *err, cudaStream_t s) {
  const int st = store ? 1 : 0;
  return with_shape(cfg, [&](auto t) {
    using S = typename decltype(t)::S;
    constexpr int CFG = decltype(t)::CFG;
    return adjoint ? launch<S, CFG, true>(sims, tiles, n_tiles, active, it, parity, st, err, s)
                   : launch<S, CFG, false>(sims, tiles, n_tiles, active, it, parity, st, err, s);
  });
}

}  // namespace tma
}  // namespace psv
