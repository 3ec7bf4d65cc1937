// Stage kernels: f64 arithmetic, RUSA Riemann solver.
#include "stage_inst.cuh"

AMR_STAGE_DEFINE(f64, rusa, amr::FLX_RUSA, double)
