// FP32 fused time step with TMA tile loads (rows padded to a multiple of 4 points).
//
// Same step as psv_fast_f32.cu -- new stresses over the tile plus a 2-point
// halo, then new velocities of the tile's own points, over ping-pong buffers
// -- but the CTA's inputs arrive by tensor-memory-access bulk copies: thread 0
// issues seven cp.async.bulk.tensor.2d loads (vx, vz with a 4-point halo;
// txx, tzz, txz, lm, mu with a 2-point halo) that complete on one mbarrier,
// and every phase then computes from shared memory. The copies zero-fill
// whatever lies outside the grid. Stresses are advanced in place in shared
// memory; lambda is lm - 2 mu.
//
// A TMA copy must start on a 16-byte boundary of the innermost (z) axis, so
// every box starts at z = Z0 - 4 (Z0 a multiple of 60, so 4 (Z0 - 4) is a
// multiple of 16) and is 68 points wide; the stress boxes use columns 2..65.
// Each warp of the compute phases owns 32 consecutive z columns and walks
// every fourth row, so column arithmetic is done once per thread.
//
// The mbarrier wait is bounded: on time-out the CTA raises the model's error
// flag, waits (bounded again) for its copies to land, and returns.
#include <cuda.h>
#include <cuda_runtime.h>

#include <cstdint>

#include "psv_fast.hpp"
#include "psv_tma.hpp"

namespace psv {
namespace tma {
namespace {

constexpr int TX = 32, TZ = 60, NT = 256;
constexpr int W = TZ + 8;          // box width (z) of every tile: Z0-4 .. Z0+TZ+4
constexpr int VR = TX + 8;         // velocity box rows (x): X0-4 .. X0+TX+4
constexpr int SR = TX + 4;         // stress / medium box rows: X0-2 .. X0+TX+2
constexpr int SC = TZ + 4;         // stress columns computed: box columns 2 .. TZ+6
constexpr int kVBytes = VR * W * 4;                      // 10880
constexpr int kSBytes = SR * W * 4;                      // 9792
constexpr int kSPitch = (kSBytes + 127) / 128 * 128;     // 128-byte aligned tile slots
constexpr int kTxBytes = 2 * kVBytes + 5 * kSBytes;      // bytes the copies deliver
constexpr int kTileBytes = 2 * kVBytes + 5 * kSPitch;
constexpr int kSmemBytes = kTileBytes + 16 + 128;        // tiles + mbarrier + alignment slack
static_assert(kVBytes % 128 == 0, "velocity tiles must stay 128-byte aligned");
static_assert(SC == 64, "two warps span the stress columns");

__device__ __forceinline__ uint32_t smem_u32(const void *p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void tma_load_2d(void *dst, const CUtensorMap *map, int c0, int c1,
                                            uint64_t *bar) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes"
      " [%0], [%1, {%2, %3}], [%4];" ::"r"(smem_u32(dst)),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(c0), "r"(c1), "r"(smem_u32(bar))
      : "memory");
}

// Bounded wait on phase `parity`: true when the phase completed.
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, uint32_t parity, uint32_t max_iter) {
  const uint32_t addr = smem_u32(bar);
  for (uint32_t i = 0; i < max_iter; ++i) {
    uint32_t done;
    asm volatile(
        "{\n .reg .pred p;\n"
        " mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3;\n"
        " selp.u32 %0, 1, 0, p;\n}"
        : "=r"(done)
        : "r"(addr), "r"(parity), "r"(1000u)
        : "memory");
    if (done) return true;
  }
  return false;
}

__device__ __forceinline__ void correlate(const fast::StepArgs &a, size_t g, float lm, float mu,
                                          float vx, float vz, float txx, float tzz, float txz) {
  const float la = lm - 2.0f * mu;
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

__device__ __forceinline__ void inject(const fast::StepArgs &a, size_t g, int gx, int gz,
                                       float b, float &vx, float &vz) {
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
__global__ void __launch_bounds__(NT, 3)
    fused_step_tma(const fast::StepArgs a, const __grid_constant__ Maps maps, int *err) {
  extern __shared__ unsigned char smem_raw[];
  unsigned char *base = reinterpret_cast<unsigned char *>(
      (reinterpret_cast<uintptr_t>(smem_raw) + 127) & ~static_cast<uintptr_t>(127));
  float(*sv)[VR][W] = reinterpret_cast<float(*)[VR][W]>(base);  // vx, vz
  auto stile = [&](int k) {  // txx tzz txz lm mu
    return reinterpret_cast<float(*)[W]>(base + 2 * kVBytes + k * kSPitch);
  };
  float(*const sxx_)[W] = stile(0);
  float(*const szz_)[W] = stile(1);
  float(*const sxz_)[W] = stile(2);
  float(*const slm)[W] = stile(3);
  float(*const smu)[W] = stile(4);
  uint64_t *bar = reinterpret_cast<uint64_t *>(base + kTileBytes);

  const int nx = a.nx, nz = a.nz, ps = a.pitch;
  const int X0 = blockIdx.y * TX, Z0 = blockIdx.x * TZ;
  const float c1 = 9.0f / 8.0f, c2 = 1.0f / 24.0f;

  if (threadIdx.x == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(1)
                 : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)),
                 "r"(kTxBytes)
                 : "memory");
    tma_load_2d(&sv[0][0][0], &maps.vx, Z0 - 4, X0 - 4, bar);
    tma_load_2d(&sv[1][0][0], &maps.vz, Z0 - 4, X0 - 4, bar);
    tma_load_2d(&sxx_[0][0], &maps.txx, Z0 - 4, X0 - 2, bar);
    tma_load_2d(&szz_[0][0], &maps.tzz, Z0 - 4, X0 - 2, bar);
    tma_load_2d(&sxz_[0][0], &maps.txz, Z0 - 4, X0 - 2, bar);
    tma_load_2d(&slm[0][0], &maps.lm, Z0 - 4, X0 - 2, bar);
    tma_load_2d(&smu[0][0], &maps.mu, Z0 - 4, X0 - 2, bar);
  }

  // While the copies fly: receivers (pre-step velocities) and this thread's
  // buoyancy values for phase C.
  if (!ADJ && a.rec_vx && blockIdx.x == 0 && blockIdx.y == 0) {
    for (int r = threadIdx.x; r < a.nr; r += NT) {
      const int c = a.rec_cell[r];
      a.rec_vx[(size_t)r * a.nt + a.it] = a.in.vx[c];
      a.rec_vz[(size_t)r * a.nt + a.it] = a.in.vz[c];
    }
  }
  // Thread layout for both compute phases: warp w covers 32 consecutive z
  // columns (half h = w & 1 of the tile) and every fourth row from q = w >> 1.
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, h = w & 1, q = w >> 1;
  constexpr int KC = TX / 4;  // own rows per thread
  const int lzc = h * 32 + lane;  // own column of this thread (valid if < TZ)
  const int gzc = Z0 + lzc;
  const bool col_ok = lzc < TZ && gzc < nz;
  float bb[KC];
#pragma unroll
  for (int k = 0; k < KC; ++k) {
    const int gx = X0 + q + 4 * k;
    bb[k] = (col_ok && gx < nx) ? __ldg(a.b + gx * ps + gzc) : 0.f;
  }

  // Bounded wait (about a second at most); the CTA agrees on the outcome so
  // that it leaves together, after its copies have landed.
  const bool landed = mbar_wait(bar, 0, 1u << 20);
  if (__syncthreads_or(!landed)) {
    if (threadIdx.x == 0) {
      atomicOr(err, 1);
      mbar_wait(bar, 0, 1u << 20);
    }
    return;
  }

  const float dtv = ADJ ? -a.dt : a.dt;
  // Phase B: new stresses over rows X0-2 .. X0+TX+2 and box columns
  // 2 .. TZ+6 (z = Z0-2 .. Z0+TZ+2), in place.
  {
    const float(*VX)[W] = sv[0];
    const float(*VZ)[W] = sv[1];
    const int c = 2 + h * 32 + lane;  // box column
    const int gz = Z0 - 4 + c;
    const bool z_in = gz >= 0 && gz < nz;
    const bool z_int = gz >= 2 && gz < nz - 2;
    const bool z_own = c >= 4 && c < TZ + 4;
    const bool z_free = gz >= a.fz0 && gz < a.fz1;
    const int tz = min(gz + 1, nz - gz);
#pragma unroll 3
    for (int k = 0; k < SR / 4; ++k) {
      const int r = q + 4 * k;  // box row
      const int gx = X0 - 2 + r;
      if (!z_in || gx < 0 || gx >= nx) continue;
      const int g = gx * nz + gz;   // unpadded (snapshots, kernels)
      const int gp = gx * ps + gz;  // padded (wave fields)
      const int vr = r + 2;  // same point in the velocity box
      float sxx = sxx_[r][c], szz = szz_[r][c], sxz = sxz_[r][c];
      const bool own = z_own && r >= 2 && r < TX + 2;
      if (own && a.snap[0]) {
        a.snap[0][g] = VX[vr][c];
        a.snap[1][g] = VZ[vr][c];
        a.snap[2][g] = sxx;
        a.snap[3][g] = szz;
        a.snap[4][g] = sxz;
      }
      const float lm = slm[r][c], mu = smu[r][c];
      if (ADJ && own && a.asnap[0] && z_free && gx >= a.fx0 && gx < a.fx1)
        correlate(a, g, lm, mu, VX[vr][c], VZ[vr][c], sxx, szz, sxz);
      if (z_int && gx >= 2 && gx < nx - 2) {
        const float la = lm - 2.0f * mu;
        const float dvx = c1 * (VX[vr + 1][c] - VX[vr][c]) + c2 * (VX[vr - 1][c] - VX[vr + 2][c]);
        const float dvz = c1 * (VZ[vr][c] - VZ[vr][c - 1]) + c2 * (VZ[vr][c - 2] - VZ[vr][c + 1]);
        const float gxz = (c1 * (VX[vr][c + 1] - VX[vr][c]) +
                           c2 * (VX[vr][c - 1] - VX[vr][c + 2])) * a.idz +
                          (c1 * (VZ[vr][c] - VZ[vr - 1][c]) +
                           c2 * (VZ[vr - 2][c] - VZ[vr + 1][c])) * a.idx;
        const float ex = dvx * a.idx, ez = dvz * a.idz;
        // Points at least np frames deep have taper exp(0) = 1 exactly.
        const int cnt = min(tz, min(gx + 1, nx - gx));
        const float tp = cnt < a.np ? __ldg(a.taper_tab + cnt) : 1.0f;
        sxx = tp * (sxx + dtv * (lm * ex + la * ez));
        szz = tp * (szz + dtv * (la * ex + lm * ez));
        sxz = tp * (sxz + dtv * mu * gxz);
        sxx_[r][c] = sxx;
        szz_[r][c] = szz;
        sxz_[r][c] = sxz;
      }
      if (own) {
        a.out.txx[gp] = sxx;
        a.out.tzz[gp] = szz;
        a.out.txz[gp] = sxz;
      }
    }
  }
  __syncthreads();

  // Phase C: new velocities of the tile's own points.
  if (col_ok) {
    const float(*TXX)[W] = sxx_;
    const float(*TZZ)[W] = szz_;
    const float(*TXZ)[W] = sxz_;
    const InjPlan &p = a.plan;
    const int c = lzc + 4;  // box column of this thread's points
    const bool z_int = gzc >= 2 && gzc < nz - 2;
    const int tz = min(gzc + 1, nz - gzc);
    const bool z_box = p.n && gzc >= p.z0 && gzc < p.z0 + p.h;
#pragma unroll
    for (int k = 0; k < KC; ++k) {
      const int lx = q + 4 * k;
      const int gx = X0 + lx;
      if (gx >= nx) continue;
      const int g = gx * nz + gzc;   // unpadded (injection cells)
      const int gp = gx * ps + gzc;  // padded
      const int r = lx + 2;  // stress box row
      float vx = sv[0][lx + 4][c], vz = sv[1][lx + 4][c];
      const float b = bb[k];
      if (z_int && gx >= 2 && gx < nx - 2) {
        const float ax = (c1 * (TXX[r][c] - TXX[r - 1][c]) + c2 * (TXX[r - 2][c] - TXX[r + 1][c])) * a.idx +
                         (c1 * (TXZ[r][c] - TXZ[r][c - 1]) + c2 * (TXZ[r][c - 2] - TXZ[r][c + 1])) * a.idz;
        const float az = (c1 * (TXZ[r + 1][c] - TXZ[r][c]) + c2 * (TXZ[r - 1][c] - TXZ[r + 2][c])) * a.idx +
                         (c1 * (TZZ[r][c + 1] - TZZ[r][c]) + c2 * (TZZ[r][c - 1] - TZZ[r][c + 2])) * a.idz;
        const int cnt = min(tz, min(gx + 1, nx - gx));
        const float tp = cnt < a.np ? __ldg(a.taper_tab + cnt) : 1.0f;
        const float bdt = b * dtv;
        vx = tp * (vx + bdt * ax);
        vz = tp * (vz + bdt * az);
      }
      if (z_box && gx >= p.x0 && gx < p.x0 + p.w) inject(a, g, gx, gzc, b, vx, vz);
      a.out.vx[gp] = vx;
      a.out.vz[gp] = vz;
    }
  }
}

template <bool ADJ>
cudaError_t launch(const fast::StepArgs &a, const Maps &maps, int *err, cudaStream_t s) {
  static unsigned long long configured = 0;
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  const unsigned long long bit = 1ull << (dev & 63);
  if (!(configured & bit)) {
    e = cudaFuncSetAttribute(fused_step_tma<ADJ>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             kSmemBytes);
    if (e != cudaSuccess) return e;
    configured |= bit;
  }
  const dim3 grid((a.nz + TZ - 1) / TZ, (a.nx + TX - 1) / TX);
  fused_step_tma<ADJ><<<grid, NT, kSmemBytes, s>>>(a, maps, err);
  return cudaGetLastError();
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

bool encode(CUtensorMap *m, const float *ptr, int nx, int nz, int pitch, int rows) {
  EncodeTiled fn = encoder();
  if (!fn) return false;
  const cuuint64_t dims[2] = {(cuuint64_t)nz, (cuuint64_t)nx};
  const cuuint64_t strides[1] = {(cuuint64_t)pitch * sizeof(float)};
  const cuuint32_t box[2] = {(cuuint32_t)W, (cuuint32_t)rows};
  const cuuint32_t elem[2] = {1, 1};
  return fn(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, const_cast<float *>(ptr), dims, strides, box,
            elem, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
            CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) ==
         CUDA_SUCCESS;
}

}  // namespace

bool supported(int nx, int nz, int pitch) {
  return pitch % 4 == 0 && pitch >= nz && nx > 0 && nz > 0 && encoder() != nullptr;
}

bool make_maps(Maps &m, const float *const fields[5], const float *lm, const float *mu, int nx,
               int nz, int pitch) {
  return encode(&m.vx, fields[0], nx, nz, pitch, VR) &&
         encode(&m.vz, fields[1], nx, nz, pitch, VR) &&
         encode(&m.txx, fields[2], nx, nz, pitch, SR) &&
         encode(&m.tzz, fields[3], nx, nz, pitch, SR) &&
         encode(&m.txz, fields[4], nx, nz, pitch, SR) && encode(&m.lm, lm, nx, nz, pitch, SR) &&
         encode(&m.mu, mu, nx, nz, pitch, SR);
}

cudaError_t forward(const SolverArgs &a, void *const second[5], int *cur, const Maps maps[2],
                    int *err, const InjPlan &plan, int shot, bool store, int it0, int it1,
                    bool zero_first, bool finish, cudaStream_t s) {
  if (zero_first) {
    const size_t bytes = (size_t)a.nx * a.pitch * sizeof(float);
    void *prim[5] = {a.vx, a.vz, a.txx, a.tzz, a.txz};
    for (int f = 0; f < 5; ++f) {
      cudaError_t e = cudaMemsetAsync(prim[f], 0, bytes, s);
      if (e == cudaSuccess) e = cudaMemsetAsync(second[f], 0, bytes, s);
      if (e != cudaSuccess) return e;
    }
    *cur = 0;
  }
  fast::StepArgs sa = fast::base_step_args(a);
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
    fast::set_step_buffers(sa, a, second, *cur);
    cudaEvent_t *ev = a.events ? a.events + 2 * (it - it0) : nullptr;
    if (ev) cudaEventRecord(ev[0], s);
    cudaError_t e = launch<false>(sa, maps[*cur], err, s);
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

cudaError_t adjoint(const SolverArgs &a, void *const second[5], int *cur, const Maps maps[2],
                    int *err, const InjPlan &plan, int shot, cudaStream_t s) {
  const size_t bytes = (size_t)a.nx * a.pitch * sizeof(float);
  void *prim[5] = {a.vx, a.vz, a.txx, a.tzz, a.txz};
  for (int f = 0; f < 5; ++f) {
    cudaError_t e = cudaMemsetAsync(prim[f], 0, bytes, s);
    if (e == cudaSuccess) e = cudaMemsetAsync(second[f], 0, bytes, s);
    if (e != cudaSuccess) return e;
  }
  *cur = 0;
  fast::StepArgs sa = fast::base_step_args(a);
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
    fast::set_step_buffers(sa, a, second, *cur);
    cudaError_t e = launch<true>(sa, maps[*cur], err, s);
    if (e != cudaSuccess) return e;
    *cur ^= 1;
  }
  return cudaGetLastError();
}

}  // namespace tma
}  // namespace psv
