// Host-side launchers of the sm_103a kernels (defined in the .cu files).
#pragma once

#include <cuda_runtime.h>

#include "amr_common.h"

namespace amr {

struct StageArgs;
struct GhostLaunch;
struct CtArgs;
struct DtArgs;
struct TreeOpArgs;
struct SplitArgs;

struct Method {
  int ng;      // ghost layers: 2, or 4 (WENO5)
  int recon;   // Recon
  int flux;    // Flux
  int f32;     // FP32 bulk storage / arithmetic
  // launch schedule (picked by Engine::autotune): threads per CTA of the
  // face-flux kernel (64 or 128), of the per-cell kernels and of the ghost fills
  int faces_block = 128;
  int cell_block = 256;
  int ghost_block = 256;
  int persistent = 0;   // face fluxes by a grid of resident CTAs looping over the face list: 1 in
                        // strides, 2 claiming 32 faces per warp from a counter (k_faces_dyn)
  // the step's kernels are launched as programmatic dependents of their
  // predecessor (each begins with pdl_wait()); AMR2D_PDL=0 turns it off
  int pdl = 1;
};

// Launches kernel `k` on stream `s`, as a programmatic dependent of the
// stream's previous kernel when `pdl` is set (the kernel must begin with
// pdl_wait()).
template <typename... KArgs, typename... Args>
inline cudaError_t launch_k(int pdl, void (*k)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t s,
                            Args... args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = grid;
  cfg.blockDim = block;
  cfg.dynamicSmemBytes = smem;
  cfg.stream = s;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  at[0].val.programmaticStreamSerializationAllowed = pdl ? 1 : 0;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, k, args...);
}

// true if the (ng, recon, flux, precision) combination is compiled
bool method_supported(const Method &m);

cudaError_t launch_stage(const Method &m, const StageArgs &a, int ntasks, cudaStream_t s);
// per-precision, per-flux entry points (one translation unit each)
#define AMR_DECL_STAGE(P, F)                                                                        \
  cudaError_t launch_stage_##P##_##F(const Method &m, const StageArgs &a, int ntasks, cudaStream_t s); \
  cudaError_t launch_faces_##P##_##F(const Method &m, const SplitArgs &a, cudaStream_t s);
AMR_DECL_STAGE(f64, rusa)
AMR_DECL_STAGE(f64, hlle)
AMR_DECL_STAGE(f64, hllc)
AMR_DECL_STAGE(f64, hlld)
AMR_DECL_STAGE(f32, rusa)
AMR_DECL_STAGE(f32, hlle)
AMR_DECL_STAGE(f32, hllc)
AMR_DECL_STAGE(f32, hlld)
#undef AMR_DECL_STAGE

// the split stage: primitive variables, face fluxes, residual + RK
cudaError_t launch_prim(const Method &m, const SplitArgs &a, cudaStream_t s);
cudaError_t launch_faces(const Method &m, const SplitArgs &a, cudaStream_t s);
cudaError_t launch_resid(const Method &m, const SplitArgs &a, cudaStream_t s);

// ghost fill: snapshot pass (if any snapshots) then the gather pass
cudaError_t launch_ghost(const Method &m, const GhostLaunch &g, cudaStream_t s);
cudaError_t launch_ct_emf(const Method &m, const CtArgs &a, int ntasks, cudaStream_t s);
cudaError_t launch_ct_face(const Method &m, const CtArgs &a, int ntasks, cudaStream_t s);
cudaError_t launch_ct_cell(const Method &m, const CtArgs &a, int ntasks, cudaStream_t s);
// the three CT kernels of a stage with fused fills, as one cooperative launch
// whose phases are separated by grid barriers (bar: two zeroed words)
struct FillFuse;
cudaError_t launch_ct_coop(const Method &m, const CtArgs &a, const FillFuse &f_emf, const FillFuse &f_face,
                           const FillFuse &f_cell, unsigned *bar, cudaStream_t s);
// diffusivity.cpp on the tasks flagged TASK_DIFFUSE (a.q = U after stage 2)
cudaError_t launch_diffuse(const Method &m, const CtArgs &a, int ntasks, cudaStream_t s);
// per-leaf max wave speed and refinement criterion from the primitive state
cudaError_t launch_dt_cell(const Method &m, const DtArgs &a, int ntasks, cudaStream_t s);
cudaError_t launch_refine(const Method &m, const TreeOpArgs &a, int nops, cudaStream_t s);
// initial condition of n root blocks (IC2Dtype.cpp + W2U), their face field and criterion
struct IcDev;
cudaError_t launch_ic(const Method &m, const IcDev *blocks, int n, const double *tabs, void *U, double *Bi,
                      double *grad, cudaStream_t s);
cudaError_t launch_coarsen(const Method &m, const TreeOpArgs &a, int nops, cudaStream_t s);

cudaError_t launch_gather(const int *slots, int nblk, const void *src, int f32, int per, double *dst,
                          cudaStream_t s);
cudaError_t launch_scatter(const int *slots, int nblk, void *dst, int f32, int per, const double *src,
                           cudaStream_t s);

}  // namespace amr
