// Stage kernels: f64 arithmetic, HLLD Riemann solver.
#include "stage_inst.cuh"

AMR_STAGE_DEFINE(f64, hlld, amr::FLX_HLLD, double)
