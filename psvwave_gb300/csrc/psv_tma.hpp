// FP32 fused time step with TMA tile loads (psv_tma_f32.cu).
#pragma once

#include <cuda.h>
#include <cuda_runtime.h>

#include "psv_solver.hpp"

namespace psv {
namespace tma {

// Tensor maps of one buffer set (the five wave fields) plus the medium.
struct Maps {
  CUtensorMap vx, vz, txx, tzz, txz, lm, mu;
};

// True when the arrays can use the TMA kernel (row pitch a multiple of 4
// points, i.e. rows on 16-byte boundaries) and the driver exposes
// tensor-map encoding.
bool supported(int nx, int nz, int pitch);

// Encodes the maps of one buffer set; false on failure.
bool make_maps(Maps &m, const float *const fields[5], const float *lm, const float *mu, int nx,
               int nz, int pitch);

// Time loops as fast::forward / fast::adjoint; maps[0] covers the primary
// buffer set, maps[1] the second. *err (device int) is raised when a CTA's
// bounded wait for its copies times out.
cudaError_t forward(const SolverArgs &a, void *const second[5], int *cur, const Maps maps[2],
                    int *err, const InjPlan &plan, int shot, bool store, int it0, int it1,
                    bool zero_first, bool finish, cudaStream_t s);
cudaError_t adjoint(const SolverArgs &a, void *const second[5], int *cur, const Maps maps[2],
                    int *err, const InjPlan &plan, int shot, cudaStream_t s);

}  // namespace tma
}  // namespace psv
