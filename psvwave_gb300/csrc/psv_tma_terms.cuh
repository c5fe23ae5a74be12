// Per-point terms shared by the FP32 fused steps (psv_tma_f32.cu,
// psv_cluster_f32.cu): the adjoint's kernel correlation with a stored
// forward snapshot (src/fdModel.cpp:817-861, FP64 accumulation) and the
// source / adjoint-source injection after the velocity update
// (src/fdModel.cpp:681-751, 951-958), in the reference's operation order.
#pragma once

#include <cuda_runtime.h>

#include "psv_tma.hpp"

namespace psv {
namespace tma {

__device__ __forceinline__ void correlate(const SimDesc &d, const float *const asnap[5], int g,
                                          float lm, float mu, float vx, float vz, float txx,
                                          float tzz, float txz) {
  const float la = lm - 2.0f * mu;
  const float avx = asnap[0][g], avz = asnap[1][g], atxx = asnap[2][g], atzz = asnap[3][g],
              atxz = asnap[4][g];
  const float r = la / lm;
  const float dd = lm - la * r;
  const float inv_den = 1.0f / (dd * dd);
  const float fxx = txx - tzz * r, fzz = tzz - txx * r;
  const float axx = atxx - atzz * r, azz = atzz - atxx * r;
  const float lam = (axx + azz) * (fxx + fzz) * inv_den;
  const float muk = (fxx * axx + fzz * azz) * inv_den + 2.0f * (txz * atxz / (4.0f * mu * mu));
  d.krho[g] -= d.sidt * static_cast<double>(avx * vx + avz * vz);
  d.klam[g] += d.sidt * static_cast<double>(lam);
  d.kmu[g] += d.sidt * 2.0 * static_cast<double>(muk);
}

__device__ __forceinline__ void inject(const SimDesc &d, int it, int g, int gx, int gz, float b,
                                       float &vx, float &vz) {
  const InjPlan &p = d.plan;
  int k = p.map[(gx - p.x0) * p.h + (gz - p.z0)];
  if (k < 0) return;
  for (; k < p.n && p.terms[k].cell == g; ++k) {
    const InjTerm t = p.terms[k];
    double term;
    if (t.kind == 0) {
      term = (((t.coef * d.stf[(size_t)t.index * d.nt + it]) * d.dt_d) * (double)b) / t.div;
    } else {
      const double *src = t.field == 0 ? d.a_ux : d.a_uz;
      term = ((d.dt_d * (double)b) * src[(size_t)t.index * d.nt + it]) / t.div;
    }
    if (t.field == 0)
      vx += (float)term;
    else
      vz += (float)term;
  }
}


}  // namespace tma
}  // namespace psv
