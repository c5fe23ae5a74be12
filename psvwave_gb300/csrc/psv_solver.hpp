// Host-side interface of the P-SV time-stepping kernels. The kernels are
// templated on the wave-field precision and compiled twice:
// psv_solver_f64.cu (double, no contraction into fused multiply-add, so the
// arithmetic is bit-identical to the reference's src/fdModel.cpp) and
// psv_solver_f32.cu (float, the production path).
#pragma once

#include <cuda_runtime.h>

#include <cstddef>

namespace psv {

// One additive term applied to a velocity point right after that point's
// velocity update (source injection src/fdModel.cpp:681-751, adjoint-source
// injection src/fdModel.cpp:951-958). Terms are kept in the reference's
// serial order; terms of one point are contiguous.
//   kind 0 (moment-tensor source):  v += (((coef * stf[index][it]) * dt) * b) / div
//   kind 1 (adjoint source):        v += ((dt * b) * a_stf[field][shot][index][it]) / div
// with coef carrying the sign of the reference's '+=' / '-='.
struct InjTerm {
  int cell;   // absolute grid index ix * nz + iz
  int field;  // 0: vx, 1: vz
  int index;  // source id (kind 0) or receiver id (kind 1)
  int kind;
  double coef;
  double div;
};

// Injection terms of one shot (or of the adjoint receivers), with a dense
// lookup table over their bounding box: map[(ix - x0) * h + (iz - z0)] is
// the first term of that point or -1.
struct InjPlan {
  int x0 = 0, z0 = 0, w = 0, h = 0;
  const int *map = nullptr;
  const InjTerm *terms = nullptr;
  int n = 0;
};

// Everything one forward or adjoint simulation of a shot touches. Pointers
// typed void are arrays of the wave-field precision T; double pointers are
// FP64 whatever T is.
struct SolverArgs {
  int nx = 0, nz = 0, nt = 0, np = 0, si = 1, snapshots = 0, nr = 0;
  int pitch = 0;  // row pitch of wave-field and medium arrays (>= nz, multiple of 4)
  double dt = 0, dx = 0, dz = 0;
  // wave fields [nx][pitch]
  void *vx = nullptr, *vz = nullptr, *txx = nullptr, *tzz = nullptr, *txz = nullptr;
  // medium: lm = lambda + 2 mu, la = lambda, mu, b = 1 / rho  [nx][pitch]
  const void *lm = nullptr, *la = nullptr, *mu = nullptr, *b = nullptr;
  // Cerjan taper by frame count, taper_tab[0..np] (src/fdModel.cpp:263-298)
  const void *taper_tab = nullptr;
  // stored forward snapshots, one array per field, [shots][snapshots][nx][nz]
  void *accu[5] = {nullptr, nullptr, nullptr, nullptr, nullptr};
  // receivers: padded cell index ix * pitch + iz, raw per-step velocities [2][nr][nt] (T)
  const int *rec_cell = nullptr;
  void *rec_raw = nullptr;
  // seismograms, FP64 [shots][nr][nt]
  double *rtf_ux = nullptr, *rtf_uz = nullptr;
  const double *a_stf_ux = nullptr, *a_stf_uz = nullptr;
  // source time functions, FP64 [n_sources][nt]
  const double *stf = nullptr;
  // Lame-basis kernels, FP64 [nx][nz]
  double *k_lam = nullptr, *k_mu = nullptr, *k_rho = nullptr;
  // free region, absolute indices [fx0, fx1) x [fz0, fz1)
  int fx0 = 0, fx1 = 0, fz0 = 0, fz1 = 0;
  // optional profiling: (launches per step + 1) events per forward time step,
  // recorded before each launch of the step and after the last one
  cudaEvent_t *events = nullptr;
};

// Time-step kernel variants. kTwoKernel: stress_step then velocity_step
// (both precisions; the FP64 path always uses it). kFused: one fused_step
// launch per time step over ping-pong buffers (FP32). kFusedTma: the same
// step with TMA tile loads (FP32, nz % 4 == 0; the default where it applies).
enum Variant {
  kFused = 0,
  kTwoKernel = 1,
  kFusedTma = 2,
  kFusedTmaPersistent = 3,
  kFusedCluster = 4
};

// Precision-specific entry points (defined in psv_solver_f32.cu / _f64.cu).
#define PSV_SOLVER_DECLS(SUFFIX)                                                          \
  cudaError_t forward_##SUFFIX(const SolverArgs &a, const InjPlan &plan, int shot,       \
                               bool store, int it0, int it1, bool zero_first,            \
                               bool finish, cudaStream_t s);                              \
  cudaError_t adjoint_##SUFFIX(const SolverArgs &a, const InjPlan &plan, int shot,       \
                               cudaStream_t s);                                           \
  cudaError_t medium_##SUFFIX(int nx, int nz, int pitch, const double *vp, const double *vs, \
                              const double *rho, void *lm, void *la, void *mu, void *b,   \
                              cudaStream_t s);                                            \
  cudaError_t unpad_##SUFFIX(int nx, int nz, int pitch, const void *src, double *dst,     \
                             cudaStream_t s);                                             \
  cudaError_t widen_##SUFFIX(size_t n, const void *src, double *dst, cudaStream_t s);    \
  cudaError_t narrow_##SUFFIX(size_t n, const double *src, void *dst, cudaStream_t s);
PSV_SOLVER_DECLS(f32)
PSV_SOLVER_DECLS(f64)
#undef PSV_SOLVER_DECLS

// One step of the exact discrete adjoint (psv_exact.cuh): from the adjoint
// state after step `it` to the state before it, accumulating the FP64 medium
// gradients. lv (vx, vz) and lt (txx, tzz, txz) are updated in place, the
// new stress adjoint goes to ot; fv holds v^it and ft tau^(it+1) of the
// forward run. Arrays are padded [nx][pitch] of the wave-field precision.
struct ExactStepArgs {
  int nx = 0, nz = 0, pitch = 0, np = 0, nt = 0, it = 0, nr = 0;
  double dt = 0, dx = 0, dz = 0;
  const void *lm = nullptr, *la = nullptr, *mu = nullptr, *b = nullptr, *taper_tab = nullptr;
  // adjoint state: l^{n+1} in (lv, lt), l^n out (ov, ot)
  const void *lv[2] = {nullptr, nullptr};
  const void *lt[3] = {nullptr, nullptr, nullptr};
  void *ov[2] = {nullptr, nullptr};
  void *ot[3] = {nullptr, nullptr, nullptr};
  const void *fv[2] = {nullptr, nullptr};
  const void *ft[3] = {nullptr, nullptr, nullptr};
  double *g_lm = nullptr, *g_la = nullptr, *g_mu = nullptr, *g_b = nullptr;
  InjPlan plan{};
  const double *stf = nullptr;
  const int *rec_cell = nullptr;           // padded receiver cells
  // Receivers grouped by cell: group g holds receivers
  // rec_order[rec_start[g] .. rec_start[g+1]) in increasing index.
  int n_rec_groups = 0;
  const int *rec_start = nullptr, *rec_order = nullptr;
  const double *adj_x = nullptr, *adj_z = nullptr;  // receiver terms [nr][nt] of the shot
};
cudaError_t exact_step_f32(const ExactStepArgs &e, cudaStream_t s);
cudaError_t exact_step_f64(const ExactStepArgs &e, cudaStream_t s);

// Seismograms from raw FP32 receiver velocities (psv_solver_f32.cu).
// With `active` non-null, nothing is written unless active[member] != 0
// (batched runs whose member set varies between replays of one graph).
cudaError_t receiver_cumsum_f32(int nr, int nt, int n_steps, double dt, double dxdz,
                                const float *raw_x, const float *raw_z, double *out_x,
                                double *out_z, cudaStream_t s, const int *active = nullptr,
                                int member = 0);

// FP64 helpers (psv_aux.cu).
cudaError_t misfit_l2(size_t n, double dt, const double *obs_ux, const double *syn_ux,
                      const double *obs_uz, const double *syn_uz, double *partials,
                      int n_partials, double *out, cudaStream_t s);
cudaError_t adjoint_sources_l2(size_t n, const double *syn_ux, const double *obs_ux,
                               const double *syn_uz, const double *obs_uz, double *a_ux,
                               double *a_uz, cudaStream_t s);
cudaError_t map_kernels(size_t n, const double *vp, const double *vs, const double *rho,
                        const double *k_lam, const double *k_mu, const double *k_rho,
                        double *vp_k, double *vs_k, double *rho_k, cudaStream_t s);
// Receiver terms of the exact adjoint: adj[r][n] = dt / (dx dz) *
// sum_{m >= n} dt (syn[r][m] - obs[r][m]), per receiver row of length nt.
cudaError_t exact_receiver_terms(int rows, int nt, double dt, double dxdz, const double *syn,
                                 const double *obs, double *adj, cudaStream_t s);
// dst[k][i] += src[k][i] for k < 3, i < n (FP64).
cudaError_t add_into3(size_t n, const double *const src[3], double *const dst[3], cudaStream_t s);
// Copies five wave-field arrays of `bytes` each (a multiple of 16, all
// pointers 16-byte aligned) from src[f] to dst[f], and to dst2[f] too when
// dst2 is non-null: one launch for a whole state.
cudaError_t copy_state(const void *const src[5], void *const dst[5], void *const *dst2,
                       size_t bytes, cudaStream_t s);
// Gradients with respect to (vp, vs, rho) from those with respect to
// (lm, la, mu, b): lm = rho vp^2, la = rho (vp^2 - 2 vs^2), mu = rho vs^2,
// b = 1 / rho.
cudaError_t exact_chain(size_t n, const double *vp, const double *vs, const double *rho,
                        const double *g_lm, const double *g_la, const double *g_mu,
                        const double *g_b, double *g_vp, double *g_vs, double *g_rho,
                        cudaStream_t s);

}  // namespace psv
