// Instantiates the stage kernel of one Riemann solver and one precision for
// every supported (ghost layers, reconstruction) pair.  Each including .cu
// file defines AMR_STAGE_PREC (f64 / f32), AMR_STAGE_T and AMR_STAGE_FLUX.
#pragma once

#include "launch.hpp"
#include "stage.cuh"
#include "stage_split.cuh"

namespace amr {

// persistent = 2 (and a.ctr set): k_stage_dyn on a grid of the CTAs the SMs
// hold at once; otherwise one CTA per leaf block
template <int NG, int RECON, int FLUX, typename S>
cudaError_t launch_stage_t(const StageArgs &a, int ntasks, int pdl, int persistent, cudaStream_t s) {
  constexpr int smem = stage_smem_bytes<NG, S>();
  constexpr int threads = StageThreads<S>::value;
  static bool attr_set = false;
  static int per_sm = 0, sms = 0;
  if (!attr_set) {
    cudaError_t e = cudaFuncSetAttribute(k_stage<NG, RECON, FLUX, S>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         smem);
    if (e == cudaSuccess)
      e = cudaFuncSetAttribute(k_stage_dyn<NG, RECON, FLUX, S>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    int dev = 0;
    if (e == cudaSuccess) e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (e == cudaSuccess)
      e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_stage_dyn<NG, RECON, FLUX, S>, threads, smem);
    if (e != cudaSuccess) return e;
    if (per_sm < 1) per_sm = 1;
    attr_set = true;
  }
  if (ntasks <= 0) return cudaSuccess;
  if (persistent == 2 && a.ctr) {
    const int grid = ntasks < sms * per_sm ? ntasks : sms * per_sm;
    return launch_k(pdl, k_stage_dyn<NG, RECON, FLUX, S>, grid, threads, smem, s, a);
  }
  return launch_k(pdl, k_stage<NG, RECON, FLUX, S>, ntasks, threads, smem, s, a);
}

template <int FLUX, typename S>
cudaError_t launch_stage_flux(const Method &m, const StageArgs &a, int ntasks, cudaStream_t s) {
  const int p = m.persistent;
  if (m.ng == 2 && m.recon == REC_MUSCL) return launch_stage_t<2, REC_MUSCL, FLUX, S>(a, ntasks, m.pdl, p, s);
  if (m.ng == 2 && m.recon == REC_WENO3) return launch_stage_t<2, REC_WENO3, FLUX, S>(a, ntasks, m.pdl, p, s);
  if (m.ng == 4 && m.recon == REC_MUSCL) return launch_stage_t<4, REC_MUSCL, FLUX, S>(a, ntasks, m.pdl, p, s);
  if (m.ng == 4 && m.recon == REC_WENO3) return launch_stage_t<4, REC_WENO3, FLUX, S>(a, ntasks, m.pdl, p, s);
  if (m.ng == 4 && m.recon == REC_WENO5) return launch_stage_t<4, REC_WENO5, FLUX, S>(a, ntasks, m.pdl, p, s);
  return cudaErrorInvalidValue;
}

#ifndef AMR_FACES_MINB
#define AMR_FACES_MINB 3
#endif

// persistent: 0 one CTA per 128 (64) faces; 1 a grid of resident CTAs
// striding over the face list; 2 the same with dynamic claims of 32 faces
// per warp (k_faces_dyn, needs a.ctr)
template <int NG, int RECON, int FLUX, typename S>
cudaError_t launch_faces_t(const SplitArgs &a, int block, int persistent, int pdl, cudaStream_t s) {
  constexpr int PER = 2 * Geo<NG>::NF * Geo<NG>::NF;
  const size_t n = static_cast<size_t>(a.ntasks) * PER;
  if (n == 0) return cudaSuccess;
  if (block != 64) block = 128;  // the kernel is bounded at 128 threads per CTA
  size_t grid = (n + block - 1) / block;
  if (persistent == 2 && !a.ctr) persistent = 1;
  if (persistent) {
    // resident CTAs per SM for each (variant, block size), looked up once
    static int per_sm[2][2] = {{0, 0}, {0, 0}}, sms = 0;
    int &ps = per_sm[persistent == 2 ? 1 : 0][block == 64 ? 0 : 1];
    if (!sms) {
      int dev = 0;
      cudaError_t e = cudaGetDevice(&dev);
      if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
      if (e != cudaSuccess) return e;
    }
    if (!ps) {
      cudaError_t e = persistent == 2
          ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(&ps, k_faces_dyn<NG, RECON, FLUX, S, AMR_FACES_MINB>,
                                                          block, 0)
          : cudaOccupancyMaxActiveBlocksPerMultiprocessor(&ps, k_faces_persist<NG, RECON, FLUX, S, AMR_FACES_MINB>,
                                                          block, 0);
      if (e != cudaSuccess) return e;
      if (ps < 1) ps = 1;
    }
    const size_t cap = static_cast<size_t>(sms) * ps;
    if (grid > cap) grid = cap;
    if (persistent == 2)
      return launch_k(pdl, k_faces_dyn<NG, RECON, FLUX, S, AMR_FACES_MINB>, static_cast<unsigned>(grid), block, 0,
                      s, a);
    return launch_k(pdl, k_faces_persist<NG, RECON, FLUX, S, AMR_FACES_MINB>, static_cast<unsigned>(grid), block, 0,
                    s, a);
  }
  return launch_k(pdl, k_faces<NG, RECON, FLUX, S, AMR_FACES_MINB>, static_cast<unsigned>(grid), block, 0, s, a);
}

template <int FLUX, typename S>
cudaError_t launch_faces_flux(const Method &m, const SplitArgs &a, cudaStream_t s) {
  const int b = m.faces_block;
  const int p = m.persistent;
  if (m.ng == 2 && m.recon == REC_MUSCL) return launch_faces_t<2, REC_MUSCL, FLUX, S>(a, b, p, m.pdl, s);
  if (m.ng == 2 && m.recon == REC_WENO3) return launch_faces_t<2, REC_WENO3, FLUX, S>(a, b, p, m.pdl, s);
  if (m.ng == 4 && m.recon == REC_MUSCL) return launch_faces_t<4, REC_MUSCL, FLUX, S>(a, b, p, m.pdl, s);
  if (m.ng == 4 && m.recon == REC_WENO3) return launch_faces_t<4, REC_WENO3, FLUX, S>(a, b, p, m.pdl, s);
  if (m.ng == 4 && m.recon == REC_WENO5) return launch_faces_t<4, REC_WENO5, FLUX, S>(a, b, p, m.pdl, s);
  return cudaErrorInvalidValue;
}

}  // namespace amr

#define AMR_STAGE_DEFINE(P, F, FLUXID, T)                                                     \
  namespace amr {                                                                          \
  cudaError_t launch_stage_##P##_##F(const Method &m, const StageArgs &a, int n, cudaStream_t s) { \
    return launch_stage_flux<FLUXID, T>(m, a, n, s);                                        \
  }                                                                                        \
  cudaError_t launch_faces_##P##_##F(const Method &m, const SplitArgs &a, cudaStream_t s) {  \
    return launch_faces_flux<FLUXID, T>(m, a, s);                                           \
  }                                                                                        \
  }
