// FP32 exact adjoint step with TMA tile loads (psv_exact_tma.cu): the same
// transpose as exact::exact_step_tile (psv_exact.cuh), with every input tile
// copied into shared memory by the tensor-memory accelerator before any
// arithmetic, and the receiver terms added in the same pass.
#pragma once

#include <cuda.h>
#include <cuda_runtime.h>

#include "psv_solver.hpp"

namespace psv {
namespace exact_tma {

// Tile: TX rows (x) by TZ columns (z).
constexpr int kTX = 16, kTZ = 32;

// Tensor maps. The adjoint state lives in one array of planes, each an
// [nx][pitch] grid (lam_v: boxes with a 4-point halo in x, lam_t: with a
// 2-point halo); the recomputed forward states in another, five planes per
// state (vx, vz, txx, tzz, txz).
struct Maps {
  CUtensorMap lam_v, lam_t, slots, lm, la, mu, b;
};

// One step n: reads l^{n+1} from planes lv[], lt[] and the forward states
// v^n (slot planes sv, sv + 1) and tau^{n+1} (slot planes st + 2 .. st + 4);
// writes l^n to olv[], olt[] (padded grids) and adds the step's terms to
// the gradient sums, float-float pairs (hi, lo) over the unpadded grid.
struct Step {
  int nx = 0, nz = 0, pitch = 0, np = 0, nt = 0, it = 0;
  float dt = 0, idx = 0, idz = 0;
  double dt_d = 0;
  const float *taper_tab = nullptr;
  int lv[2] = {0, 0}, lt[3] = {0, 0, 0}, sv = 0, st = 0;
  float *olv[2] = {nullptr, nullptr};
  float *olt[3] = {nullptr, nullptr, nullptr};
  float2 *g_lm = nullptr, *g_la = nullptr, *g_mu = nullptr, *g_b = nullptr;
  // Optional FP32 partial sums per point of the padded grid (index
  // ix * pitch + iz): g_part_lmu holds (lm, mu), g_part_b holds b. The
  // step's terms are added there, and on a flush step the partial plus the
  // terms go into the pairs and the partial is reset to 0. With partial
  // sums, lambda's term is folded into lm's and mu's (the FP32 forward
  // forms lambda = lm - 2 mu, so these are the gradients of its inputs):
  // g_la stays untouched. Null: every step adds the four terms into the
  // pairs directly.
  float2 *g_part_lmu = nullptr;
  float *g_part_b = nullptr;
  int flush = 1;
  InjPlan plan{};
  const double *stf = nullptr;
  // Receivers by tile (tiles row-major over ceil(nz / kTZ) columns): tile t
  // holds receivers rec_list[rec_start[t] .. rec_start[t + 1]) in increasing
  // index; rec_cell are padded cells, adj_x / adj_z the shot's terms [nr][nt].
  const int *rec_cell = nullptr, *rec_start = nullptr, *rec_list = nullptr;
  const double *adj_x = nullptr, *adj_z = nullptr;
  int *err = nullptr;  // raised when a CTA's bounded wait for its copies times out
};

// Encodes the maps: `lam` holds n_lam planes, `slots` n_slot_planes planes,
// plane_bytes apart. False on failure.
bool encode(Maps &m, const float *lam, int n_lam, const float *slots, int n_slot_planes,
            size_t plane_bytes, const float *lm, const float *la, const float *mu, const float *b,
            int nx, int nz, int pitch);

// Tile index of cell (ix, iz).
int tile_of(int nz, int ix, int iz);
int tile_count(int nx, int nz);

cudaError_t step(const Maps &maps, const Step &a, cudaStream_t s);

// out[k][i] = hi + lo of the pair ff[k][i] in FP64, k = 0..3, i < n.
cudaError_t finish(size_t n, float2 *const ff[4], double *const out[4], cudaStream_t s);
// out[k][i] += hi + lo of ff[k][i] in FP64 (out[k][i] = ... when `first`).
cudaError_t accumulate(size_t n, const float2 *const ff[4], double *const out[4], bool first,
                       cudaStream_t s);

}  // namespace exact_tma
}  // namespace psv
