// Surrogate network kernels (forward, backward, Adam) and the coarse-to-grid
// parameter map of the Monte Carlo workload; see psv_cnn.hpp.
//
// The convolutions run on the tensor cores as tcgen05 implicit GEMMs with
// BF16 hi + lo operand splits and FP32 accumulators in TMEM: the forward
// and the input gradient (with the ReLU mask of the layer's input fused in)
// in conv_tc, the weight and bias gradients in conv_weight_tc as
// fixed-order partial sums over position ranges that a second kernel adds
// up, so every result is deterministic.
#include "psv_cnn.hpp"

#include <algorithm>
#include <cmath>
#include <vector>

#include "../../include/psvwave.h"

namespace psv {
namespace cnn {

namespace {

constexpr int kThreads = 256;

size_t layer_size(int l) { return (size_t)kCout[l] * kCin[l] * 9 + kCout[l]; }


__device__ __forceinline__ void tap(int k, int dil, int &dh, int &dc) {
  dh = (k / 3 - 1) * dil;
  dc = (k % 3 - 1) * dil;
}

// ---- tensor-core convolutions (tcgen05): forward and input gradient -------
//
// The forward convolution as an implicit GEMM on the 5th-generation tensor
// cores: D[pos][co] = sum_k A[pos][k] W[co][k], with pos = b kP + p running
// over the batch (kTcM = 128 positions per CTA, the MMA's M), co over the
// output channels (N = cout rounded up to 16), and k = ci * 9 + tap over
// the input channels and the 3 x 3 taps. K runs in chunks of kTcKc = 64:
// seven input channels (63 columns) and one zero column, so that a column's
// channel and tap are compile-time constants of the unrolled gather. Per
// chunk each of the 128 threads gathers its position's row of the im2col
// tile into shared memory (16-byte stores) as two BF16 matrices,
// hi = bf16(x) and lo = bf16(x - hi), and the threads copy the chunk of
// BF16 weights; one thread issues the tcgen05.mma instructions
// (kind::f16, BF16 x BF16 -> FP32) for both, accumulating into a TMEM tile
// of 128 lanes x 64 columns, and commits them to an mbarrier that every
// thread waits on (bounded) before the next chunk overwrites the tiles.
// Each warp then reads its 32 TMEM lanes (tcgen05.ld), adds the bias,
// applies the ReLU and writes y[b][co][p].
//
// The hi + lo split keeps 16 significant bits of each activation (about
// 2^-17 relative; the products of BF16 values are exact in FP32), so the
// results are the FP32 convolution of the activations so rounded, up to
// accumulation order: BF16 weights, FP32 activations and accumulation, as
// the network is specified, to about 1e-6 relative.
//
// Shared-memory operands are K-major without swizzle: 8 x 16-byte core
// matrices, element (r, k) at (r / 8) * kTcSBO + (k / 8) * 128 +
// (r % 8) * 16 + (k % 8) * 2; the descriptor's leading byte offset (between
// K-adjacent core matrices) is 128, its stride byte offset (between 8-row
// groups) kTcSBO.
constexpr int kTcM = 128, kTcKc = 64, kTcCi = 7, kTcThreads = 128, kTcCols = 64;
constexpr int kTcLBO = 128, kTcSBO = (kTcKc / 8) * 128;

__device__ __forceinline__ uint32_t tc_saddr(const void *p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}
__device__ __forceinline__ int tc_off(int r, int k) {
  return (r >> 3) * kTcSBO + (k >> 3) * kTcLBO + (r & 7) * 16 + (k & 7) * 2;
}
// Shared-memory matrix descriptor: start address >> 4 (bits 0-13), leading
// byte offset >> 4 (16-29), stride byte offset >> 4 (32-45), descriptor
// version 1 (bit 46), no swizzle (61-63 = 0).
__device__ __forceinline__ uint64_t tc_desc(uint32_t addr) {
  return (uint64_t)((addr & 0x3FFFF) >> 4) | ((uint64_t)(kTcLBO >> 4) << 16) |
         ((uint64_t)(kTcSBO >> 4) << 32) | ((uint64_t)1 << 46);
}
__device__ __forceinline__ void tc_mma(uint32_t tmem, uint64_t a, uint64_t b, uint32_t idesc,
                                       uint32_t accumulate) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}" ::"r"(tmem),
      "l"(a), "l"(b), "r"(idesc), "r"(accumulate)
      : "memory");
}
__device__ __forceinline__ bool tc_wait(uint32_t bar, uint32_t parity) {
  for (uint32_t i = 0; i < (1u << 20); ++i) {
    uint32_t done;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3;\n"
        " selp.u32 %0, 1, 0, p;\n}"
        : "=r"(done)
        : "r"(bar), "r"(parity), "r"(1000u)
        : "memory");
    if (done) return true;
  }
  return false;
}

// MODE kFwdRelu / kFwdLinear: the forward convolution above (x = layer
// input [B][cin][kP], y = output [B][cout][kP], bias added, ReLU or not).
// MODE kBwdData: the input gradient dx[b][ci][p] = (sum_co sum_tap
// w[co][ci][tap] dy[b][co][p - off_tap]) [act[b][ci][p] > 0] as the same
// implicit GEMM with the roles of the channels swapped: x = dy (gathered at
// the negated tap offsets, K = cout * 9), B[ci][co * 9 + tap] =
// w[co][ci][tap], N = cin rounded up to 16, and the ReLU mask of the
// layer's input activation `act` applied in the epilogue (bias unused).
constexpr int kFwdRelu = 0, kFwdLinear = 1, kBwdData = 2;

template <int MODE>
__global__ void __launch_bounds__(kTcThreads) conv_tc(int batch, int cin_l, int cout_l, int npad,
                                                     int dil, const float *__restrict__ x,
                                                     const __nv_bfloat16 *__restrict__ w,
                                                     const float *__restrict__ bias,
                                                     const float *__restrict__ act,
                                                     float *__restrict__ y, int *err) {
  constexpr bool BWD = MODE == kBwdData;
  // Channels gathered (the GEMM's K / 9) and produced (its N).
  const int cin = BWD ? cout_l : cin_l, cout = BWD ? cin_l : cout_l;
  __shared__ __align__(1024) unsigned char a_hi[kTcM * kTcKc * 2];
  __shared__ __align__(1024) unsigned char a_lo[kTcM * kTcKc * 2];
  __shared__ __align__(1024) unsigned char b_w[kTcCols * kTcKc * 2];
  __shared__ __align__(8) uint64_t bar;
  __shared__ uint32_t tmem_holder;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int total = batch * kP, pos0 = blockIdx.x * kTcM;
  const int K = cin * 9;
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     tc_saddr(&tmem_holder)),
                 "r"(kTcCols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  if (tid == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(tc_saddr(&bar)), "r"(1)
                 : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  // This thread's position for the gather (row tid of the tile) and the
  // offsets of its nine taps within an input channel (-1 outside the image).
  const int pos = pos0 + tid;
  const bool row_ok = pos < total;
  const int bs = row_ok ? pos / kP : 0, ps = row_ok ? pos - bs * kP : 0;
  const int h = ps / kW, c = ps - h * kW;
  int nb[9];
#pragma unroll
  for (int t = 0; t < 9; ++t) {
    int dh, dc;
    tap(t, dil, dh, dc);
    const int hh = BWD ? h - dh : h + dh, cc = BWD ? c - dc : c + dc;
    nb[t] = (row_ok && hh >= 0 && hh < kH && cc >= 0 && cc < kW) ? hh * kW + cc : -1;
  }
  const float *xb = x + (size_t)bs * cin * kP;
  // idesc: D FP32 (bits 4-5 = 1), A and B BF16 (7-9 = 1, 10-12 = 1), both
  // K-major, N >> 3 (17-22), M >> 4 (24-28).
  const uint32_t idesc = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(npad >> 3) << 17) |
                         ((uint32_t)(kTcM >> 4) << 24);
  bool ok = true;
  uint32_t tmem = 0;
  int ch = 0;
  const int chunks = (cin + kTcCi - 1) / kTcCi;
  for (; ch < chunks; ++ch) {
    const int ci0 = ch * kTcCi;
#pragma unroll
    for (int g = 0; g < kTcKc / 8; ++g) {
      uint32_t hi2[4], lo2[4];
#pragma unroll
      for (int e = 0; e < 8; e += 2) {
        float v[2];
#pragma unroll
        for (int q = 0; q < 2; ++q) {
          const int kk = 8 * g + e + q, j = kk / 9, t = kk - 9 * (kk / 9);
          v[q] = 0.f;
          if (kk < 9 * kTcCi && ci0 + j < cin && nb[t] >= 0)
            v[q] = __ldg(xb + (size_t)(ci0 + j) * kP + nb[t]);
        }
        const __nv_bfloat162 h2 = __floats2bfloat162_rn(v[0], v[1]);
        const float2 hf = __bfloat1622float2(h2);
        const __nv_bfloat162 l2 = __floats2bfloat162_rn(v[0] - hf.x, v[1] - hf.y);
        hi2[e / 2] = *reinterpret_cast<const uint32_t *>(&h2);
        lo2[e / 2] = *reinterpret_cast<const uint32_t *>(&l2);
      }
      *reinterpret_cast<uint4 *>(a_hi + tc_off(tid, 8 * g)) =
          make_uint4(hi2[0], hi2[1], hi2[2], hi2[3]);
      *reinterpret_cast<uint4 *>(a_lo + tc_off(tid, 8 * g)) =
          make_uint4(lo2[0], lo2[1], lo2[2], lo2[3]);
    }
    for (int i = tid; i < npad * kTcKc; i += kTcThreads) {
      const int co = i / kTcKc, kk = i - co * kTcKc, k = ci0 * 9 + kk;
      __nv_bfloat16 v = __float2bfloat16_rn(0.f);
      if (co < cout && kk < 9 * kTcCi && k < K) {
        // Forward: w[co][k]. Input gradient: row co is the layer's input
        // channel, k = (output channel, tap) of the layer.
        v = BWD ? w[((size_t)(k / 9) * cout + co) * 9 + (k - 9 * (k / 9))]
                : w[(size_t)co * K + k];
      }
      *reinterpret_cast<__nv_bfloat16 *>(b_w + tc_off(co, kk)) = v;
    }
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    tmem = tmem_holder;
    if (tid == 0) {
      for (int s = 0; s < kTcKc / 16; ++s) {
        const uint32_t koff = s * 2 * kTcLBO;
        const uint64_t bd = tc_desc(tc_saddr(b_w) + koff);
        tc_mma(tmem, tc_desc(tc_saddr(a_hi) + koff), bd, idesc, (ch > 0 || s > 0) ? 1u : 0u);
        tc_mma(tmem, tc_desc(tc_saddr(a_lo) + koff), bd, idesc, 1u);
      }
      asm volatile(
          "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
              tc_saddr(&bar))
          : "memory");
    }
    // The chunk's products must be done before its tiles are overwritten.
    if (!tc_wait(tc_saddr(&bar), (uint32_t)(ch & 1))) ok = false;
    if (__syncthreads_or(!ok)) {
      ok = false;
      break;
    }
  }
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  if (ok) {
    const int row = 32 * warp + lane, g = pos0 + row;
    const bool valid = g < total;
    const int b = valid ? g / kP : 0, p = valid ? g - b * kP : 0;
    for (int c0 = 0; c0 < npad; c0 += 16) {
      uint32_t v[16];
      const uint32_t ta = tmem + ((uint32_t)(32 * warp) << 16) + (uint32_t)c0;
      asm volatile(
          "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,"
          "%14,%15}, [%16];"
          : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]),
            "=r"(v[7]), "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]),
            "=r"(v[13]), "=r"(v[14]), "=r"(v[15])
          : "r"(ta));
      asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
      if (valid) {
#pragma unroll
        for (int j = 0; j < 16; ++j) {
          const int co = c0 + j;
          if (co < cout) {
            const size_t o = ((size_t)b * cout + co) * kP + p;
            if (BWD) {
              y[o] = act[o] > 0.f ? __uint_as_float(v[j]) : 0.f;
            } else {
              float r = __uint_as_float(v[j]) + bias[co];
              if (MODE == kFwdRelu) r = fmaxf(r, 0.f);
              y[o] = r;
            }
          }
        }
      }
    }
  } else if (tid == 0) {
    atomicOr(err, 1);
    // Bounded: give the products of the chunk that timed out (the last ones
    // issued) more time to finish before the TMEM is freed.
    tc_wait(tc_saddr(&bar), (uint32_t)(ch & 1));
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 0)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem),
                 "r"(kTcCols)
                 : "memory");
}

// ---- tensor-core weight gradients (tcgen05) --------------------------------
//
// dW[co][k] = sum_pos dy[pos][co] X[pos][k] and db[co] = sum_pos dy[pos][co]
// as a GEMM whose reduction runs over the positions pos = b kP + p of the
// batch: D[k][co] (M = 128 rows of k = ci * 9 + tap per CTA, the bias as row
// k = cin * 9 with X = 1; N = cout rounded up to 16) accumulates
// A[k][pos] B[co][pos] over chunks of 64 positions, with A = X^T the
// transposed im2col of the layer input and B = dy^T. Both operands are FP32
// values split into BF16 hi + lo parts; hi.hi + hi.lo + lo.hi (three
// tcgen05.mma kind::f16 per 16 positions) carry the products to about 2^-16
// relative, the FP32 accumulation order is fixed, and blockIdx.y splits the
// chunks into kChunks ranges whose partial sums sum_chunks adds in order
// (deterministic). Per chunk thread t gathers position t % 64 of rows
// (t / 64) * 64 .. + 63 of A and every other row of B, one thread issues
// the MMAs and commits them to an mbarrier every thread waits on (bounded;
// a time-out raises the error flag). The epilogue reads row 32 w + lane of
// the accumulator (tcgen05.ld.32x32b) and writes the CTA's partial sums in
// the layout of the weights ((co cin + ci) 9 + tap, then the biases).
__global__ void __launch_bounds__(kTcThreads) conv_weight_tc(int batch, int cin, int cout,
                                                            int npad, int dil,
                                                            const float *__restrict__ x,
                                                            const float *__restrict__ dy,
                                                            float *__restrict__ partial, int *err) {
  __shared__ __align__(1024) unsigned char a_hi[kTcM * kTcKc * 2];
  __shared__ __align__(1024) unsigned char a_lo[kTcM * kTcKc * 2];
  __shared__ __align__(1024) unsigned char b_hi[kTcCols * kTcKc * 2];
  __shared__ __align__(1024) unsigned char b_lo[kTcCols * kTcKc * 2];
  __shared__ __align__(8) uint64_t bar;
  __shared__ uint32_t tmem_holder;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int K = cin * 9;  // weight columns; row K is the bias
  const int m0 = blockIdx.x * kTcM;
  const int total = batch * kP;
  const int n_chunks = (total + kTcKc - 1) / kTcKc;
  const int c0 = (int)((long long)n_chunks * blockIdx.y / gridDim.y);
  const int c1 = (int)((long long)n_chunks * (blockIdx.y + 1) / gridDim.y);
  const size_t len = (size_t)cout * K + cout;
  float *out = partial + (size_t)blockIdx.y * len;
  const int k_out = m0 + 32 * warp + lane;  // the accumulator row this thread writes
  auto out_index = [&](int co) {
    return k_out < K ? (size_t)co * K + k_out : (size_t)cout * K + co;
  };
  if (c0 >= c1) {  // no positions in this range: zero partial sums
    if (k_out <= K)
      for (int co = 0; co < cout; ++co) out[out_index(co)] = 0.f;
    return;
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     tc_saddr(&tmem_holder)),
                 "r"(kTcCols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  if (tid == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(tc_saddr(&bar)), "r"(1)
                 : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  const uint32_t idesc = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(npad >> 3) << 17) |
                         ((uint32_t)(kTcM >> 4) << 24);
  const int j = tid & 63, half = tid >> 6;
  bool ok = true;
  uint32_t tmem = 0;
  int ch = c0;
  for (; ch < c1; ++ch) {
    const int g = ch * kTcKc + j;
    const bool valid = g < total;
    const int b = valid ? g / kP : 0, p = valid ? g - b * kP : 0;
    const int h = p / kW, c = p - h * kW;
    const float *xb = x + (size_t)b * cin * kP;
    // A: rows half * 64 .. + 63 at position column j.
    int k = m0 + half * 64;
    int ci = k / 9, t = k - 9 * ci;
    for (int mm = 0; mm < 64; ++mm, ++k) {
      float v = 0.f;
      if (k < K) {
        int dh, dc;
        tap(t, dil, dh, dc);
        const int hh = h + dh, cc = c + dc;
        if (valid && hh >= 0 && hh < kH && cc >= 0 && cc < kW)
          v = __ldg(xb + (size_t)ci * kP + hh * kW + cc);
      } else if (k == K) {
        v = valid ? 1.f : 0.f;
      }
      const __nv_bfloat16 vh = __float2bfloat16_rn(v);
      const __nv_bfloat16 vl = __float2bfloat16_rn(v - __bfloat162float(vh));
      *reinterpret_cast<__nv_bfloat16 *>(a_hi + tc_off(half * 64 + mm, j)) = vh;
      *reinterpret_cast<__nv_bfloat16 *>(a_lo + tc_off(half * 64 + mm, j)) = vl;
      if (++t == 9) {
        t = 0;
        ++ci;
      }
    }
    // B: rows co = half, half + 2, ... at position column j.
    for (int co = half; co < npad; co += 2) {
      const float v =
          (valid && co < cout) ? __ldg(dy + ((size_t)b * cout + co) * kP + p) : 0.f;
      const __nv_bfloat16 vh = __float2bfloat16_rn(v);
      const __nv_bfloat16 vl = __float2bfloat16_rn(v - __bfloat162float(vh));
      *reinterpret_cast<__nv_bfloat16 *>(b_hi + tc_off(co, j)) = vh;
      *reinterpret_cast<__nv_bfloat16 *>(b_lo + tc_off(co, j)) = vl;
    }
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    tmem = tmem_holder;
    if (tid == 0) {
      for (int s = 0; s < kTcKc / 16; ++s) {
        const uint32_t koff = s * 2 * kTcLBO;
        const uint64_t ah = tc_desc(tc_saddr(a_hi) + koff), al = tc_desc(tc_saddr(a_lo) + koff);
        const uint64_t bh = tc_desc(tc_saddr(b_hi) + koff), bl = tc_desc(tc_saddr(b_lo) + koff);
        tc_mma(tmem, ah, bh, idesc, (ch > c0 || s > 0) ? 1u : 0u);
        tc_mma(tmem, ah, bl, idesc, 1u);
        tc_mma(tmem, al, bh, idesc, 1u);
      }
      asm volatile(
          "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
              tc_saddr(&bar))
          : "memory");
    }
    // The chunk's products must be done before its tiles are overwritten.
    if (!tc_wait(tc_saddr(&bar), (uint32_t)((ch - c0) & 1))) ok = false;
    if (__syncthreads_or(!ok)) {
      ok = false;
      break;
    }
  }
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  if (ok) {
    for (int col = 0; col < npad; col += 16) {
      uint32_t v[16];
      const uint32_t ta = tmem + ((uint32_t)(32 * warp) << 16) + (uint32_t)col;
      asm volatile(
          "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,"
          "%14,%15}, [%16];"
          : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]),
            "=r"(v[7]), "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]),
            "=r"(v[13]), "=r"(v[14]), "=r"(v[15])
          : "r"(ta));
      asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
      if (k_out <= K) {
#pragma unroll
        for (int q = 0; q < 16; ++q)
          if (col + q < cout) out[out_index(col + q)] = __uint_as_float(v[q]);
      }
    }
  } else if (tid == 0) {
    atomicOr(err, 1);
    // Bounded: give the products of the chunk that timed out more time to
    // finish before the TMEM is freed.
    tc_wait(tc_saddr(&bar), (uint32_t)((ch - c0) & 1));
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 0)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem),
                 "r"(kTcCols)
                 : "memory");
}

__global__ void sum_chunks(size_t len, const float *__restrict__ partial, float *__restrict__ out) {
  const size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (i >= len) return;
  float s = 0.f;
  for (int c = 0; c < kChunks; ++c) s += partial[(size_t)c * len + i];
  out[i] = s;
}

// Fixed-order block sum of kThreads values.
__device__ float block_sum(float v, float *red) {
  red[threadIdx.x] = v;
  __syncthreads();
  for (int s = kThreads / 2; s > 0; s >>= 1) {
    if ((int)threadIdx.x < s) red[threadIdx.x] += red[threadIdx.x + s];
    __syncthreads();
  }
  const float r = red[0];
  __syncthreads();
  return r;
}

__device__ float misfit_of(const float *yb, float *red) {
  float s = 0.f;
  for (int p = threadIdx.x; p < kP; p += kThreads) s += yb[3 * kP + p];
  return block_sum(s, red);
}

// Loss = w_m mean_b (m - m*)^2 + w_g mean_{b,c,p} (g - g*)^2 and its
// gradient with respect to the last layer's output.
__global__ void __launch_bounds__(kThreads) head_loss(int batch, const float *__restrict__ y4,
                                                      const float *__restrict__ m_true,
                                                      const float *__restrict__ g_true, float w_m,
                                                      float w_g, float *__restrict__ dy4,
                                                      double *__restrict__ loss_part) {
  __shared__ float red[kThreads];
  const int b = blockIdx.x;
  const float *yb = y4 + (size_t)b * 4 * kP;
  const float m = misfit_of(yb, red);
  const float dm = m - m_true[b];
  const float ng = (float)batch * 3 * kP;
  float lg = 0.f;
  for (int i = threadIdx.x; i < 3 * kP; i += kThreads) {
    const float diff = yb[i] - g_true[(size_t)b * 3 * kP + i];
    lg += diff * diff;
    dy4[(size_t)b * 4 * kP + i] = 2.f * w_g * diff / ng;
  }
  for (int p = threadIdx.x; p < kP; p += kThreads)
    dy4[(size_t)b * 4 * kP + 3 * kP + p] = 2.f * w_m * dm / (float)batch;
  lg = block_sum(lg, red);
  if (threadIdx.x == 0)
    loss_part[b] = (double)w_m * dm * dm / batch + (double)w_g * lg / ng;
}

__global__ void sum_loss(int n, const double *__restrict__ part, double *__restrict__ out) {
  if (threadIdx.x == 0 && blockIdx.x == 0) {
    double s = 0;
    for (int i = 0; i < n; ++i) s += part[i];
    *out = s;
  }
}

__global__ void __launch_bounds__(kThreads) head_predict(const float *__restrict__ y4,
                                                         float *__restrict__ misfit,
                                                         float *__restrict__ grad) {
  __shared__ float red[kThreads];
  const int b = blockIdx.x;
  const float *yb = y4 + (size_t)b * 4 * kP;
  const float m = misfit_of(yb, red);
  for (int i = threadIdx.x; i < 3 * kP; i += kThreads) grad[(size_t)b * 3 * kP + i] = yb[i];
  if (threadIdx.x == 0) misfit[b] = m;
}

__global__ void adam_step(size_t n, float *__restrict__ p, const float *__restrict__ g,
                          float *__restrict__ m, float *__restrict__ v,
                          __nv_bfloat16 *__restrict__ wbf, float lr, float b1, float b2, float eps,
                          float bc1, float bc2) {
  const size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float gi = g[i];
  const float mi = b1 * m[i] + (1.f - b1) * gi;
  const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
  m[i] = mi;
  v[i] = vi;
  const float pi = p[i] - lr * (mi / bc1) / (sqrtf(vi / bc2) + eps);
  p[i] = pi;
  wbf[i] = __float2bfloat16_rn(pi);
}

__global__ void to_bf16(size_t n, const float *__restrict__ p, __nv_bfloat16 *__restrict__ wbf) {
  const size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (i < n) wbf[i] = __float2bfloat16_rn(p[i]);
}

unsigned blocks(size_t n, int t = 256) { return static_cast<unsigned>((n + t - 1) / t); }

void check(cudaError_t e, const char *what) { cuda_check(e, what); }

}  // namespace

size_t weight_offset(int layer) {
  size_t off = 0;
  for (int l = 0; l < layer; ++l) off += layer_size(l);
  return off;
}

size_t bias_offset(int layer) { return weight_offset(layer) + (size_t)kCout[layer] * kCin[layer] * 9; }

size_t num_params() { return weight_offset(kLayers); }

Net::Net(int device, int max_batch) : device_(device), max_batch_(max_batch) {
  if (max_batch <= 0) throw Error(PSV_ERR_INVALID_ARGUMENT, "max_batch must be positive");
  DeviceGuard guard(device_);
  check(cudaStreamCreateWithFlags(&stream_, cudaStreamNonBlocking), "cudaStreamCreate");
  const size_t n = num_params();
  params_.allocate(n * sizeof(float));
  wbf_.allocate(n * sizeof(__nv_bfloat16));
  grads_.allocate(n * sizeof(float));
  adam_m_.allocate(n * sizeof(float));
  adam_v_.allocate(n * sizeof(float));
  size_t maxlen = 0;
  for (int l = 0; l < kLayers; ++l) maxlen = std::max(maxlen, layer_size(l));
  partials_.allocate(kChunks * maxlen * sizeof(float));
  for (int l = 0; l < kLayers; ++l)
    act_[l].allocate((size_t)max_batch * kCout[l] * kP * sizeof(float));
  for (auto &d : dact_) d.allocate((size_t)max_batch * kMaxC * kP * sizeof(float));
  loss_partials_.allocate((size_t)max_batch * sizeof(double));
  loss_.allocate(sizeof(double));
  err_.allocate(sizeof(int));
  check(cudaMemset(err_.get(), 0, sizeof(int)), "err flag");
}

// Raises when a tensor-core convolution's bounded wait for its products
// timed out (the flag is cleared for the next call).
void Net::check_error() {
  int flag = 0;
  check(cudaMemcpyAsync(&flag, err_.get(), sizeof(int), cudaMemcpyDeviceToHost, stream_), "err");
  check(cudaStreamSynchronize(stream_), "err");
  if (flag) {
    check(cudaMemsetAsync(err_.get(), 0, sizeof(int), stream_), "err");
    throw Error(PSV_ERR_CUDA, "a tensor-core convolution timed out waiting for its products");
  }
}

Net::~Net() {
  if (stream_) {
    int prev = 0;
    cudaGetDevice(&prev);
    cudaSetDevice(device_);
    cudaStreamSynchronize(stream_);
    cudaStreamDestroy(stream_);
    cudaSetDevice(prev);
  }
}

void Net::check_batch(int batch) const {
  if (batch <= 0 || batch > max_batch_)
    throw Error(PSV_ERR_INVALID_ARGUMENT, "batch must be in [1, max_batch]");
}

void Net::refresh_bf16() {
  const size_t n = num_params();
  to_bf16<<<blocks(n), 256, 0, stream_>>>(n, params_.as<float>(), wbf_.as<__nv_bfloat16>());
  check(cudaGetLastError(), "to_bf16");
}

void Net::set_params(const float *host) {
  DeviceGuard guard(device_);
  const size_t n = num_params();
  check(cudaMemcpyAsync(params_.get(), host, n * sizeof(float), cudaMemcpyHostToDevice, stream_),
        "set params");
  check(cudaMemsetAsync(adam_m_.get(), 0, n * sizeof(float), stream_), "adam");
  check(cudaMemsetAsync(adam_v_.get(), 0, n * sizeof(float), stream_), "adam");
  step_ = 0;
  refresh_bf16();
  check(cudaStreamSynchronize(stream_), "set params");
}

void Net::get_params(float *host) {
  DeviceGuard guard(device_);
  check(cudaMemcpyAsync(host, params_.get(), num_params() * sizeof(float), cudaMemcpyDeviceToHost,
                        stream_),
        "get params");
  check(cudaStreamSynchronize(stream_), "get params");
}

void Net::forward(int batch, const float *x) {
  const float *in = x;
  for (int l = 0; l < kLayers; ++l) {
    const __nv_bfloat16 *w = wbf_.as<__nv_bfloat16>() + weight_offset(l);
    const float *bias = params_.as<float>() + bias_offset(l);
    float *out = act_[l].as<float>();
    const int npad = std::max(16, (kCout[l] + 15) / 16 * 16);
    const unsigned tiles = static_cast<unsigned>((batch * kP + kTcM - 1) / kTcM);
    if (l + 1 < kLayers)
      conv_tc<kFwdRelu><<<tiles, kTcThreads, 0, stream_>>>(
          batch, kCin[l], kCout[l], npad, kDil[l], in, w, bias, nullptr, out, err_.as<int>());
    else
      conv_tc<kFwdLinear><<<tiles, kTcThreads, 0, stream_>>>(
          batch, kCin[l], kCout[l], npad, kDil[l], in, w, bias, nullptr, out, err_.as<int>());
    check(cudaGetLastError(), "conv forward");
    in = out;
  }
}

double Net::backward(int batch, const float *x, const float *m_true, const float *g_true,
                     float w_misfit, float w_grad) {
  float *cur = dact_[0].as<float>(), *other = dact_[1].as<float>();
  head_loss<<<batch, kThreads, 0, stream_>>>(batch, act_[kLayers - 1].as<float>(), m_true, g_true,
                                             w_misfit, w_grad, cur, loss_partials_.as<double>());
  sum_loss<<<1, 32, 0, stream_>>>(batch, loss_partials_.as<double>(), loss_.as<double>());
  check(cudaGetLastError(), "head loss");
  for (int l = kLayers - 1; l >= 0; --l) {
    const float *in = l == 0 ? x : act_[l - 1].as<float>();
    const int rows = kCin[l] * 9 + 1;  // weights of one output channel, then its bias
    const unsigned mtiles = static_cast<unsigned>((rows + kTcM - 1) / kTcM);
    conv_weight_tc<<<dim3(mtiles, kChunks), kTcThreads, 0, stream_>>>(
        batch, kCin[l], kCout[l], std::max(16, (kCout[l] + 15) / 16 * 16), kDil[l], in, cur,
        partials_.as<float>(), err_.as<int>());
    const size_t len = layer_size(l);
    sum_chunks<<<blocks(len), 256, 0, stream_>>>(len, partials_.as<float>(),
                                                 grads_.as<float>() + weight_offset(l));
    check(cudaGetLastError(), "conv backward weight");
    if (l > 0) {
      const unsigned tiles = static_cast<unsigned>((batch * kP + kTcM - 1) / kTcM);
      conv_tc<kBwdData><<<tiles, kTcThreads, 0, stream_>>>(
          batch, kCin[l], kCout[l], std::max(16, (kCin[l] + 15) / 16 * 16), kDil[l], cur,
          wbf_.as<__nv_bfloat16>() + weight_offset(l), nullptr, act_[l - 1].as<float>(), other,
          err_.as<int>());
      check(cudaGetLastError(), "conv backward data");
      std::swap(cur, other);
    }
  }
  double loss = 0;
  check(cudaMemcpyAsync(&loss, loss_.get(), sizeof(double), cudaMemcpyDeviceToHost, stream_),
        "loss");
  check(cudaStreamSynchronize(stream_), "backward");
  check_error();
  return loss;
}

void Net::predict(int batch, const float *x, float *misfit, float *grad) {
  check_batch(batch);
  DeviceGuard guard(device_);
  forward(batch, x);
  head_predict<<<batch, kThreads, 0, stream_>>>(act_[kLayers - 1].as<float>(), misfit, grad);
  check(cudaGetLastError(), "head predict");
  check(cudaStreamSynchronize(stream_), "predict");
  check_error();
}

double Net::loss_grad(int batch, const float *x, const float *m_true, const float *g_true,
                      float w_misfit, float w_grad, float *dparams_host) {
  check_batch(batch);
  DeviceGuard guard(device_);
  forward(batch, x);
  const double loss = backward(batch, x, m_true, g_true, w_misfit, w_grad);
  if (dparams_host) {
    check(cudaMemcpyAsync(dparams_host, grads_.get(), num_params() * sizeof(float),
                          cudaMemcpyDeviceToHost, stream_),
          "grads");
    check(cudaStreamSynchronize(stream_), "grads");
  }
  return loss;
}

double Net::train_step(int batch, const float *x, const float *m_true, const float *g_true,
                       float w_misfit, float w_grad, const Adam &opt) {
  check_batch(batch);
  DeviceGuard guard(device_);
  forward(batch, x);
  const double loss = backward(batch, x, m_true, g_true, w_misfit, w_grad);
  ++step_;
  const float bc1 = 1.f - std::pow(opt.beta1, (float)step_);
  const float bc2 = 1.f - std::pow(opt.beta2, (float)step_);
  const size_t n = num_params();
  adam_step<<<blocks(n), 256, 0, stream_>>>(n, params_.as<float>(), grads_.as<float>(),
                                            adam_m_.as<float>(), adam_v_.as<float>(),
                                            wbf_.as<__nv_bfloat16>(), opt.lr, opt.beta1, opt.beta2,
                                            opt.eps, bc1, bc2);
  check(cudaGetLastError(), "adam");
  return loss;
}

}  // namespace cnn

// ---- coarse-to-grid map ---------------------------------------------------

namespace {

__global__ void coarse_to_fields(int batch, int nx, int nz, int ncx, int ncz,
                                 const int *__restrict__ x0, const int *__restrict__ x1,
                                 const double *__restrict__ wx, const int *__restrict__ z0,
                                 const int *__restrict__ z1, const double *__restrict__ wz,
                                 const double *__restrict__ mean, const double *__restrict__ sigma,
                                 const float *__restrict__ z, double *__restrict__ fields) {
  const size_t n = (size_t)batch * 3 * nx * nz;
  const size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int iz = (int)(i % nz);
  const int ix = (int)((i / nz) % nx);
  const int c = (int)((i / ((size_t)nx * nz)) % 3);
  const int b = (int)(i / ((size_t)3 * nx * nz));
  const size_t cb = (size_t)c * ncx * ncz;
  const float *zb = z + (size_t)b * 3 * ncx * ncz + cb;
  auto theta = [&](int a, int d) {
    const size_t k = (size_t)a * ncz + d;
    return mean[cb + k] + sigma[cb + k] * (double)zb[k];
  };
  const double fx = wx[ix], fz = wz[iz];
  const int a0 = x0[ix], a1 = x1[ix], d0 = z0[iz], d1 = z1[iz];
  fields[i] = (1.0 - fx) * ((1.0 - fz) * theta(a0, d0) + fz * theta(a0, d1)) +
              fx * ((1.0 - fz) * theta(a1, d0) + fz * theta(a1, d1));
}

__global__ void fields_to_coarse(int nx, int nz, int ncx, int ncz, const int *__restrict__ x0,
                                 const int *__restrict__ x1, const double *__restrict__ wx,
                                 const int *__restrict__ z0, const int *__restrict__ z1,
                                 const double *__restrict__ wz, const int *__restrict__ xs,
                                 const int *__restrict__ xe, const int *__restrict__ zs,
                                 const int *__restrict__ ze, const double *__restrict__ sigma,
                                 double scale, const double *__restrict__ g,
                                 float *__restrict__ gz) {
  const int bc = blockIdx.x;  // b * 3 + c
  const int c = bc % 3;
  const double *gb = g + (size_t)bc * nx * nz;
  for (int k = threadIdx.x; k < ncx * ncz; k += blockDim.x) {
    const int a = k / ncz, d = k - a * ncz;
    double acc = 0;
    for (int ix = xs[a]; ix < xe[a]; ++ix) {
      const double ax = (x0[ix] == a ? 1.0 - wx[ix] : 0.0) + (x1[ix] == a ? wx[ix] : 0.0);
      if (ax == 0.0) continue;
      double row = 0;
      for (int iz = zs[d]; iz < ze[d]; ++iz) {
        const double az = (z0[iz] == d ? 1.0 - wz[iz] : 0.0) + (z1[iz] == d ? wz[iz] : 0.0);
        row += az * gb[(size_t)ix * nz + iz];
      }
      acc += ax * row;
    }
    gz[(size_t)bc * ncx * ncz + k] =
        (float)(scale * sigma[(size_t)c * ncx * ncz + k] * acc);
  }
}

// 1-D interpolation weights and supports along one axis of n fine points
// (np boundary frames each side) over nc coarse nodes.
void axis_weights(int n, int np, int nc, std::vector<int> &i0, std::vector<int> &i1,
                  std::vector<double> &w, std::vector<int> &s, std::vector<int> &e) {
  const int inner = n - 2 * np;
  const double f = static_cast<double>(inner) / nc;
  i0.resize(n);
  i1.resize(n);
  w.resize(n);
  s.assign(nc, n);
  e.assign(nc, 0);
  for (int x = 0; x < n; ++x) {
    const int xi = std::min(std::max(x - np, 0), inner - 1);
    double u = (xi + 0.5) / f - 0.5;
    u = std::min(std::max(u, 0.0), static_cast<double>(nc - 1));
    int a = static_cast<int>(std::floor(u));
    a = std::min(a, nc - 1);
    i0[x] = a;
    i1[x] = std::min(a + 1, nc - 1);
    w[x] = u - a;
    for (int k : {i0[x], i1[x]}) {
      s[k] = std::min(s[k], x);
      e[k] = std::max(e[k], x + 1);
    }
  }
}

template <class V>
void upload(DeviceBuffer &d, const V &v) {
  d.allocate(std::max<size_t>(v.size(), 1) * sizeof(v[0]));
  if (!v.empty())
    cuda_check(cudaMemcpy(d.get(), v.data(), v.size() * sizeof(v[0]), cudaMemcpyHostToDevice),
               "upload coarse map");
}

}  // namespace

CoarseMap::CoarseMap(int device, int nx_, int nz_, int np_, int ncx_, int ncz_, const double *mean,
                     const double *sigma)
    : nx(nx_), nz(nz_), np(np_), ncx(ncx_), ncz(ncz_), device_(device) {
  if (nx <= 2 * np || nz <= 2 * np || ncx <= 0 || ncz <= 0 || ncx > nx - 2 * np ||
      ncz > nz - 2 * np)
    throw Error(PSV_ERR_INVALID_ARGUMENT, "coarse grid does not fit the inner grid");
  DeviceGuard guard(device_);
  std::vector<int> x0, x1, xs, xe, z0, z1, zs, ze;
  std::vector<double> wx, wz;
  axis_weights(nx, np, ncx, x0, x1, wx, xs, xe);
  axis_weights(nz, np, ncz, z0, z1, wz, zs, ze);
  upload(x0_, x0);
  upload(x1_, x1);
  upload(wx_, wx);
  upload(z0_, z0);
  upload(z1_, z1);
  upload(wz_, wz);
  upload(xs_, xs);
  upload(xe_, xe);
  upload(zs_, zs);
  upload(ze_, ze);
  const size_t n = (size_t)3 * ncx * ncz;
  upload(mean_, std::vector<double>(mean, mean + n));
  upload(sigma_, std::vector<double>(sigma, sigma + n));
  cuda_check(cudaStreamCreateWithFlags(&stream_, cudaStreamNonBlocking), "cudaStreamCreate");
}

CoarseMap::~CoarseMap() {
  if (stream_) {
    int prev = 0;
    cudaGetDevice(&prev);
    cudaSetDevice(device_);
    cudaStreamSynchronize(stream_);
    cudaStreamDestroy(stream_);
    cudaSetDevice(prev);
  }
}

void CoarseMap::to_fields(int batch, const float *z, double *fields, cudaStream_t s) const {
  DeviceGuard guard(device_);
  const size_t n = (size_t)batch * 3 * nx * nz;
  if (!n) return;
  cudaStream_t use = s ? s : stream_;
  coarse_to_fields<<<static_cast<unsigned>((n + 255) / 256), 256, 0, use>>>(
      batch, nx, nz, ncx, ncz, x0_.as<int>(), x1_.as<int>(), wx_.as<double>(), z0_.as<int>(),
      z1_.as<int>(), wz_.as<double>(), mean_.as<double>(), sigma_.as<double>(), z, fields);
  cuda_check(cudaGetLastError(), "coarse to fields");
  if (!s) cuda_check(cudaStreamSynchronize(stream_), "coarse to fields");
}

void CoarseMap::gradient(int batch, const double *gfields, float *gz, double scale,
                         cudaStream_t s) const {
  DeviceGuard guard(device_);
  if (batch <= 0) return;
  cudaStream_t use = s ? s : stream_;
  fields_to_coarse<<<batch * 3, 256, 0, use>>>(nx, nz, ncx, ncz, x0_.as<int>(), x1_.as<int>(),
                                               wx_.as<double>(), z0_.as<int>(), z1_.as<int>(),
                                               wz_.as<double>(), xs_.as<int>(), xe_.as<int>(),
                                               zs_.as<int>(), ze_.as<int>(), sigma_.as<double>(),
                                               scale, gfields, gz);
  cuda_check(cudaGetLastError(), "fields to coarse");
  if (!s) cuda_check(cudaStreamSynchronize(stream_), "fields to coarse");
}

}  // namespace psv
