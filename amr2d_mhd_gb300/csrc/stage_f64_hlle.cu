// Stage kernels: f64 arithmetic, HLLE Riemann solver.
#include "stage_inst.cuh"

AMR_STAGE_DEFINE(f64, hlle, amr::FLX_HLLE, double)
