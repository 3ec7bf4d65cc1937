// Stage kernels: f32 arithmetic, HLLD Riemann solver.
#include "stage_inst.cuh"

AMR_STAGE_DEFINE(f32, hlld, amr::FLX_HLLD, float)
