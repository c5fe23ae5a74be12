// Double-precision wave fields: the reference's own precision. Built with
// -fmad=false so that no multiply-add is fused and every operation rounds as
// the reference's double code does (src/fdModel.cpp).
#include "psv_exact.cuh"
#include "psv_kernels.cuh"

PSV_DEFINE_SOLVER(double, f64)
PSV_DEFINE_EXACT(double, f64)
