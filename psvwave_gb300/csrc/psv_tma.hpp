// FP32 fused time step with TMA tile loads (psv_tma_f32.cu), for one or many
// simulations per launch.
//
// A *simulation* is one shot of one model: its wave-field buffer sets, its
// medium, receivers, injection terms and (per shot) snapshot block. Every
// launch advances every simulation of a table by one time step; the CTAs of
// the launch are the tiles of all simulations, listed in a tile table. A
// single model's shot is a table of one.
#pragma once

#include <cuda.h>
#include <cuda_runtime.h>

#include <vector>

#include "psv_fast.hpp"
#include "psv_solver.hpp"

namespace psv {
namespace tma {

// Tensor maps of one buffer set (the five wave fields) plus the medium.
struct Maps {
  CUtensorMap vx, vz, txx, tzz, txz, lm, mu;
};

// Tile shapes (x rows by z columns, threads per CTA).
enum TileCfg { kTile32x60 = 0, kTile16x28 = 1, kTile20x28 = 2, kTile16x60 = 3, kNumTileCfgs = 4 };
void tile_dims(int cfg, int *tx, int *tz);

// Everything a CTA needs about its simulation; lives in device memory.
struct alignas(128) SimDesc {
  Maps maps[2];                // tensor maps for the descriptor's tile shape; parity p reads set p
  fast::Fields set[2];         // wave-field buffer sets
  int nx = 0, nz = 0, pitch = 0, np = 0, nt = 0, nr = 0, si = 1;
  float dt = 0, idx = 0, idz = 0;
  double dt_d = 0;
  const float *lm = nullptr, *b = nullptr, *taper_tab = nullptr;
  const float *mu = nullptr;  // (the TMA steps read mu through the maps)
  float *accu[5] = {nullptr, nullptr, nullptr, nullptr, nullptr};  // this shot's snapshots
  double *krho = nullptr, *klam = nullptr, *kmu = nullptr;
  double sidt = 0;
  int fx0 = 0, fx1 = 0, fz0 = 0, fz1 = 0;
  const int *rec_cell = nullptr;  // padded cells
  float *rec_vx = nullptr, *rec_vz = nullptr;  // [nr][nt]
  InjPlan plan{};                 // forward: sources of the shot; adjoint: receivers
  const double *stf = nullptr, *a_ux = nullptr, *a_uz = nullptr;
  // Receivers by tile of this descriptor's tile shape (tiles row-major over
  // ceil(nz / TZ) tile columns): tile t holds receivers
  // rec_list[rec_start[t] .. rec_start[t + 1]). Used by the persistent step.
  const int *rec_start = nullptr, *rec_list = nullptr;
  // Position of this simulation's tiles in a batch's tile table (row-major,
  // tiles_z columns) for the persistent batched step.
  int tile_base = 0, tiles_x = 0, tiles_z = 0;
};

// True when tensor-map encoding is available and the row pitch is a
// multiple of 4 points (16-byte rows).
bool supported(int nx, int nz, int pitch);

// A 2-D tensor map over an [nx][pitch] float array (nz valid columns) with
// width x rows boxes; a 3-D one over `planes` such arrays plane_bytes apart
// (boxes one plane deep). False on failure.
bool encode_2d(CUtensorMap *m, const float *ptr, int nx, int nz, int pitch, int width, int rows);
bool encode_planes(CUtensorMap *m, const float *base, int planes, size_t plane_bytes, int nx,
                   int nz, int pitch, int width, int rows);

// Encodes desc.maps for tile shape `cfg` from desc.set, desc.lm and the mu
// array; false on failure.
bool make_maps(SimDesc &desc, const float *mu, int cfg);
// Encodes the tensor maps that read the wave-field set `in` (with the medium
// lm, mu) for tile shape `cfg`; false on failure.
bool encode_input_maps(Maps &m, const fast::Fields &in, const float *lm, const float *mu, int nx,
                       int nz, int pitch, int cfg);

// Appends the tiles of simulation `sim` (one int4 per CTA: sim, x0, z0,
// first-tile flag) for tile shape `cfg`.
void append_tiles(int cfg, int sim, int nx, int nz, std::vector<int4> &tiles);

// One time step of every simulation in `sims` (device table), over the
// tiles in `tiles` (device, n_tiles entries); with `active` (device, one
// flag per simulation) non-null, only simulations flagged non-zero step.
// parity p: inputs in set p, outputs in set 1 - p. store: forward snapshots
// at steps it % si == 0. *err is raised when a CTA's bounded wait for its
// copies times out.
cudaError_t step(const SimDesc *sims, const int4 *tiles, int n_tiles, const int *active, int cfg,
                 bool adjoint, int it, int parity, bool store, int *err, cudaStream_t s);

// The same step for one simulation whose descriptor `desc` goes out whole
// as a kernel parameter; tiles follow from the grid.
cudaError_t step_single(const SimDesc &desc, int cfg, bool adjoint, int it, int parity,
                        bool store, int *err, cudaStream_t s);

// n_steps time steps of one simulation in a single persistent launch: steps
// it0, it0 + 1, ... (forward) or it0, it0 - 1, ... (adjoint), the first
// reading set `parity0`. CTAs take (step, tile) items in step-major order
// from a counter and start an item once the neighbouring tiles have
// finished the previous step, so no step waits for the whole grid. `sched`
// is device scratch of sched_words(...) zeroed words; errors (a timed-out
// copy or dependency wait) raise *err.
size_t sched_words(int cfg, int nx, int nz);
cudaError_t steps_persistent(const SimDesc &desc, int cfg, bool adjoint, int it0, int n_steps,
                             int parity0, bool store, int *err, unsigned *sched, cudaStream_t s);
// n_steps time steps of every simulation of a batch in one persistent
// launch, over the batch's tile table (each simulation's tiles contiguous,
// row-major, at sims[s].tile_base); with `active` non-null only flagged
// simulations step. sched: sched_words_batch(n_tiles) zeroed words.
size_t sched_words_batch(int n_tiles);
cudaError_t steps_persistent_batch(const SimDesc *sims, const int4 *tiles, int n_tiles,
                                   const int *active, int cfg, int n_steps, bool store, int *err,
                                   unsigned *sched, cudaStream_t s);
// Number of tiles of tile shape cfg over an nx x nz grid, and the tile of
// point (ix, iz).
int tile_count(int cfg, int nx, int nz);
// CTAs of the persistent step of tile shape cfg that fit on the current
// device at once (0 if the query fails).
int resident_ctas(int cfg, bool adjoint);
int tile_of(int cfg, int nz, int ix, int iz);

}  // namespace tma
}  // namespace psv
