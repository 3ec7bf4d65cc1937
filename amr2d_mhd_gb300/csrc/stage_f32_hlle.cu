// Stage kernels: f32 arithmetic, HLLE Riemann solver.
#include "stage_inst.cuh"

AMR_STAGE_DEFINE(f32, hlle, amr::FLX_HLLE, float)
