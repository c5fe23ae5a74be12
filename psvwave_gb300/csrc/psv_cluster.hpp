// FP32 time stepping of a small grid held entirely in the shared memory of
// one thread-block cluster (psv_cluster_f32.cu).
//
// The cluster's CTAs split the grid into slabs of whole x rows. Each CTA
// keeps its rows of the five wave fields, plus two halo rows on each side,
// and its rows of lm, mu and b, in shared memory for every time step of
// the launch. After each half-step it writes the two edge rows it computed
// into its neighbours' halo rows (distributed shared memory), and the
// cluster barrier orders the half-steps. Global memory carries only the
// initial and final state, receivers, snapshots, correlations and
// injection. Same arithmetic, in the same order, as the TMA steps
// (psv_tma_f32.cu).
#pragma once

#include <cuda_runtime.h>

#include "psv_tma.hpp"

namespace psv {
namespace cluster {

// The cluster size (CTAs) that holds an nx x nz grid with np taper frames,
// or 0 when none does: 16 (non-portable) or 8 CTAs, each of at most the
// device's opt-in shared memory, at least two rows per CTA, and a cluster
// the device can place. Sets the kernels' launch attributes as a side
// effect (call outside stream capture).
int plan(int nx, int nz, int np);

// n_steps steps of simulation d from set `parity` (forward: it0, it0 + 1,
// ...; adjoint: it0, it0 - 1, ...), final state in set parity ^ (n_steps & 1);
// forward snapshots when store. One launch of `nc` CTAs (nc from plan).
cudaError_t steps(const tma::SimDesc &d, bool adjoint, int it0, int n_steps, int parity,
                  bool store, int nc, cudaStream_t s);

// Batched forward: the cluster size for members of sizes nx[k] x nz[k]
// (np[k] frames), k < n, each in its own cluster (the largest member's
// shared memory per CTA, returned in *smem), or 0 when one does not fit.
// Sets the batch kernel's launch attributes (call outside stream capture).
int plan_batch(const int *nx, const int *nz, const int *np, int n, size_t *smem);

// Forward steps 0 .. n_steps - 1 of the n simulations of the device table
// `sims`, from set 0 (final state in set n_steps & 1), one cluster of nc
// CTAs each, in one launch; with `active` non-null only members flagged
// non-zero run.
cudaError_t steps_batch(const tma::SimDesc *sims, const int *active, int n, int nc, size_t smem,
                        int n_steps, bool store, cudaStream_t s);

}  // namespace cluster
}  // namespace psv
