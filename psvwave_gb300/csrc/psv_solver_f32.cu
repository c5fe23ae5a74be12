// Single-precision wave fields: the production path. Seismograms, misfit and
// kernel sums stay FP64.
#include "psv_kernels.cuh"

PSV_DEFINE_SOLVER(float, f32)
