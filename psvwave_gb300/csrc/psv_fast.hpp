// FP32 fused time step (psv_fast_f32.cu): arguments and time-loop drivers.
#pragma once

#include <cuda_runtime.h>

#include "psv_solver.hpp"

namespace psv {
namespace fast {

struct Fields {
  float *vx, *vz, *txx, *tzz, *txz;
};
struct ConstFields {
  const float *vx, *vz, *txx, *tzz, *txz;
};

struct StepArgs {
  int nx = 0, nz = 0, np = 0, nt = 0, it = 0;
  int pitch = 0;  // row pitch of wave-field and medium arrays
  float dt = 0, idx = 0, idz = 0;  // time step, 1/dx, 1/dz
  double dt_d = 0;
  ConstFields in{};
  Fields out{};
  const float *lm = nullptr, *la = nullptr, *mu = nullptr, *b = nullptr;
  const float *taper_tab = nullptr;
  // forward snapshot destination (null: no snapshot this step)
  float *snap[5] = {nullptr, nullptr, nullptr, nullptr, nullptr};
  // adjoint: stored snapshot to correlate with (null: not a snapshot step)
  const float *asnap[5] = {nullptr, nullptr, nullptr, nullptr, nullptr};
  double *krho = nullptr, *klam = nullptr, *kmu = nullptr;
  double sidt = 0;
  int fx0 = 0, fx1 = 0, fz0 = 0, fz1 = 0;
  // receivers (forward): pre-step velocities into [nr][nt] buffers
  const int *rec_cell = nullptr;
  float *rec_vx = nullptr, *rec_vz = nullptr;
  int nr = 0;
  // injection terms of the step
  InjPlan plan{};
  const double *stf = nullptr, *a_ux = nullptr, *a_uz = nullptr;
};

cudaError_t step(const StepArgs &a, bool adjoint, cudaStream_t s);

// StepArgs fields that do not change within a simulation.
StepArgs base_step_args(const SolverArgs &a);
// Points in/out at the buffer set holding the current state (cur: 0 =
// primary, 1 = second) and at the other one.
void set_step_buffers(StepArgs &s, const SolverArgs &a, void *const second[5], int cur);

// Time loops over two buffer sets: `primary` = the SolverArgs fields,
// `second` = the other set. *cur (0 = primary, 1 = second) names the set that
// holds the current state and is updated as the loop swaps them. Events, if
// requested in SolverArgs::events, are recorded before and after each step's
// single launch (two per step).
cudaError_t forward(const SolverArgs &a, void *const second[5], int *cur, const InjPlan &plan,
                    int shot, bool store, int it0, int it1, bool zero_first, bool finish,
                    cudaStream_t s);
cudaError_t adjoint(const SolverArgs &a, void *const second[5], int *cur, const InjPlan &plan,
                    int shot, cudaStream_t s);

}  // namespace fast
}  // namespace psv
