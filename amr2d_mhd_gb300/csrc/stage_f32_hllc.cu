// Stage kernels: f32 arithmetic, HLLC Riemann solver.
#include "stage_inst.cuh"

AMR_STAGE_DEFINE(f32, hllc, amr::FLX_HLLC, float)
