// Stage kernels: f64 arithmetic, HLLC Riemann solver.
#include "stage_inst.cuh"

AMR_STAGE_DEFINE(f64, hllc, amr::FLX_HLLC, double)
