// Stage kernels: f32 arithmetic, RUSA Riemann solver.
#include "stage_inst.cuh"

AMR_STAGE_DEFINE(f32, rusa, amr::FLX_RUSA, float)
