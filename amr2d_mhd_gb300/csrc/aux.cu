// Launchers of the ghost-fill, CT, dt / criterion and refine / coarsen
// kernels, and the stage dispatcher.  Compiled without FMA contraction: the
// FP64 instantiations reproduce the reference's arithmetic.
#include "aux_kernels.cuh"
#include "launch.hpp"
#include "stage_split.cuh"

namespace amr {

bool method_supported(const Method &m) {
  if (m.flux < FLX_RUSA || m.flux > FLX_HLLD) return false;
  if (m.ng == 2) return m.recon == REC_MUSCL || m.recon == REC_WENO3;
  if (m.ng == 4) return m.recon == REC_MUSCL || m.recon == REC_WENO3 || m.recon == REC_WENO5;
  return false;
}

cudaError_t launch_stage(const Method &m, const StageArgs &a, int n, cudaStream_t s) {
  if (!method_supported(m)) return cudaErrorInvalidValue;
  if (!m.f32) {
    switch (m.flux) {
      case FLX_RUSA: return launch_stage_f64_rusa(m, a, n, s);
      case FLX_HLLE: return launch_stage_f64_hlle(m, a, n, s);
      case FLX_HLLC: return launch_stage_f64_hllc(m, a, n, s);
      default: return launch_stage_f64_hlld(m, a, n, s);
    }
  }
  switch (m.flux) {
    case FLX_RUSA: return launch_stage_f32_rusa(m, a, n, s);
    case FLX_HLLE: return launch_stage_f32_hlle(m, a, n, s);
    case FLX_HLLC: return launch_stage_f32_hllc(m, a, n, s);
    default: return launch_stage_f32_hlld(m, a, n, s);
  }
}

cudaError_t launch_faces(const Method &m, const SplitArgs &a, cudaStream_t s) {
  if (!method_supported(m)) return cudaErrorInvalidValue;
  if (!m.f32) {
    switch (m.flux) {
      case FLX_RUSA: return launch_faces_f64_rusa(m, a, s);
      case FLX_HLLE: return launch_faces_f64_hlle(m, a, s);
      case FLX_HLLC: return launch_faces_f64_hllc(m, a, s);
      default: return launch_faces_f64_hlld(m, a, s);
    }
  }
  switch (m.flux) {
    case FLX_RUSA: return launch_faces_f32_rusa(m, a, s);
    case FLX_HLLE: return launch_faces_f32_hlle(m, a, s);
    case FLX_HLLC: return launch_faces_f32_hllc(m, a, s);
    default: return launch_faces_f32_hlld(m, a, s);
  }
}

namespace {
int cell_threads(const Method &m) { return m.cell_block == 128 || m.cell_block == 512 ? m.cell_block : 256; }
}  // namespace

cudaError_t launch_prim(const Method &m, const SplitArgs &a, cudaStream_t s) {
  const int nn = m.ng == 2 ? Geo<2>::NN : Geo<4>::NN;
  const size_t n = static_cast<size_t>(a.ntasks) * nn;
  if (n == 0) return cudaSuccess;
  if (a.fuse.apply.nseg) {  // fused fill: one CTA per leaf
    if (m.ng == 2 && !m.f32) return launch_k(m.pdl, k_prim_task<2, double>, a.ntasks, 256, 0, s, a);
    if (m.ng == 2) return launch_k(m.pdl, k_prim_task<2, float>, a.ntasks, 256, 0, s, a);
    if (!m.f32) return launch_k(m.pdl, k_prim_task<4, double>, a.ntasks, 256, 0, s, a);
    return launch_k(m.pdl, k_prim_task<4, float>, a.ntasks, 256, 0, s, a);
  }
  const int b = cell_threads(m);
  const unsigned g = static_cast<unsigned>((n + b - 1) / b);
  if (m.ng == 2 && !m.f32) return launch_k(m.pdl, k_prim<2, double>, g, b, 0, s, a);
  if (m.ng == 2) return launch_k(m.pdl, k_prim<2, float>, g, b, 0, s, a);
  if (!m.f32) return launch_k(m.pdl, k_prim<4, double>, g, b, 0, s, a);
  return launch_k(m.pdl, k_prim<4, float>, g, b, 0, s, a);
}

cudaError_t launch_resid(const Method &m, const SplitArgs &a, cudaStream_t s) {
  const int nn = m.ng == 2 ? Geo<2>::NN : Geo<4>::NN;
  const size_t n = static_cast<size_t>(a.ntasks) * 8 * nn;
  if (n == 0) return cudaSuccess;
  const int b = cell_threads(m);
  const unsigned g = static_cast<unsigned>((n + b - 1) / b);
  if (m.ng == 2 && !m.f32) return launch_k(m.pdl, k_resid<2, double>, g, b, 0, s, a);
  if (m.ng == 2) return launch_k(m.pdl, k_resid<2, float>, g, b, 0, s, a);
  if (!m.f32) return launch_k(m.pdl, k_resid<4, double>, g, b, 0, s, a);
  return launch_k(m.pdl, k_resid<4, float>, g, b, 0, s, a);
}

cudaError_t launch_ghost(const Method &m, const GhostLaunch &in, cudaStream_t s) {
  const int B = m.ghost_block == 128 || m.ghost_block == 512 ? m.ghost_block : 256;
  const int ng = m.ng;
  GhostLaunch g = in;
  g.row0[0] = 0;
  for (int q = 0; q < g.nseg; q++) g.row0[q + 1] = g.row0[q] + g.seg[q].nv;
  const unsigned rows = static_cast<unsigned>(g.row0[g.nseg]);
  const dim3 gs((g.nsnaps + B - 1) / B, rows), go((g.nops + B - 1) / B, rows);
  if (g.nsnaps > 0 && rows > 0) {
    const cudaError_t e = ng == 2 ? launch_k(m.pdl, k_ghost_snap<Geo<2>::N>, gs, B, 0, s, g)
                                  : launch_k(m.pdl, k_ghost_snap<Geo<4>::N>, gs, B, 0, s, g);
    if (e != cudaSuccess) return e;
  }
  if (g.nops > 0 && rows > 0)
    return ng == 2 ? launch_k(m.pdl, k_ghost_apply<Geo<2>::N>, go, B, 0, s, g)
                   : launch_k(m.pdl, k_ghost_apply<Geo<4>::N>, go, B, 0, s, g);
  return cudaSuccess;
}

#define AMR_DISPATCH_NG_S(m, KERNEL, grid, block, smem, s, args)                 \
  do {                                                                            \
    if ((m).ng == 2 && !(m).f32) KERNEL<2, double><<<grid, block, smem, s>>>(args); \
    else if ((m).ng == 2) KERNEL<2, float><<<grid, block, smem, s>>>(args);       \
    else if (!(m).f32) KERNEL<4, double><<<grid, block, smem, s>>>(args);         \
    else KERNEL<4, float><<<grid, block, smem, s>>>(args);                        \
  } while (0)

// the same for the step's kernels, as programmatic dependents (Method::pdl)
#define AMR_DISPATCH_NG_S_PDL(m, KERNEL, grid, block, smem, s, args)                                          \
  (((m).ng == 2 && !(m).f32) ? launch_k((m).pdl, KERNEL<2, double>, dim3(grid), dim3(block), smem, s, args) \
   : ((m).ng == 2)           ? launch_k((m).pdl, KERNEL<2, float>, dim3(grid), dim3(block), smem, s, args)  \
   : !(m).f32                ? launch_k((m).pdl, KERNEL<4, double>, dim3(grid), dim3(block), smem, s, args) \
                             : launch_k((m).pdl, KERNEL<4, float>, dim3(grid), dim3(block), smem, s, args))

cudaError_t launch_ct_emf(const Method &m, const CtArgs &a, int n, cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  return AMR_DISPATCH_NG_S_PDL(m, k_ct_emf, n, 128, 0, s, a);
}

cudaError_t launch_ct_face(const Method &m, const CtArgs &a, int n, cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  return m.ng == 2 ? launch_k(m.pdl, k_ct_face<2>, n, 128, 0, s, a) : launch_k(m.pdl, k_ct_face<4>, n, 128, 0, s, a);
}

// one cooperative launch (all CTAs resident: grid = SMs x resident CTAs per
// SM, capped at the task count), not a programmatic dependent
cudaError_t launch_ct_coop(const Method &m, const CtArgs &a, const FillFuse &f_emf, const FillFuse &f_face,
                           const FillFuse &f_cell, unsigned *bar, cudaStream_t s) {
  if (a.ntasks <= 0) return cudaSuccess;
  // 128 threads per CTA: 256 measured 3 % slower on the FP32 batches, 64
  // 1-3 % slower on the FP32 64-rotor batch and the FP64 rotor
  static int per_sm[2][2] = {{0, 0}, {0, 0}}, sms = 0;
  const int gi = m.ng == 2 ? 0 : 1, si = m.f32 ? 1 : 0;
#ifndef AMR_CT_COOP_THREADS
#define AMR_CT_COOP_THREADS 128
#endif
  constexpr int threads = AMR_CT_COOP_THREADS;
  void (*k)(CtArgs, FillFuse, FillFuse, FillFuse, unsigned *) =
      m.ng == 2 ? (m.f32 ? k_ct_coop<2, float, threads> : k_ct_coop<2, double, threads>)
                : (m.f32 ? k_ct_coop<4, float, threads> : k_ct_coop<4, double, threads>);
  if (!sms) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (e != cudaSuccess) return e;
  }
  int &ps = per_sm[gi][si];
  if (!ps) {
    cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&ps, k, threads, 0);
    if (e != cudaSuccess) return e;
    if (ps < 1) return cudaErrorInvalidConfiguration;
  }
  const int cap = sms * ps;
  const int grid = a.ntasks < cap ? a.ntasks : cap;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(grid);
  cfg.blockDim = dim3(threads);
  cfg.dynamicSmemBytes = 0;
  cfg.stream = s;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeCooperative;
  at[0].val.cooperative = 1;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, k, a, f_emf, f_face, f_cell, bar);
}

cudaError_t launch_diffuse(const Method &m, const CtArgs &a, int n, cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  return AMR_DISPATCH_NG_S_PDL(m, k_diffuse, n, 128, 0, s, a);
}

cudaError_t launch_ct_cell(const Method &m, const CtArgs &a, int n, cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  return AMR_DISPATCH_NG_S_PDL(m, k_ct_cell, n, 128, 0, s, a);
}

cudaError_t launch_dt_cell(const Method &m, const DtArgs &a, int n, cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  return AMR_DISPATCH_NG_S_PDL(m, k_dt_cell, n, 256, 0, s, a);
}

cudaError_t launch_ic(const Method &m, const IcDev *blocks, int n, const double *tabs, void *U, double *Bi,
                      double *grad, cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  if (m.ng == 2 && !m.f32) k_ic<2, double><<<n, 256, 0, s>>>(blocks, tabs, static_cast<double *>(U), Bi, grad);
  else if (m.ng == 2) k_ic<2, float><<<n, 256, 0, s>>>(blocks, tabs, static_cast<float *>(U), Bi, grad);
  else if (!m.f32) k_ic<4, double><<<n, 256, 0, s>>>(blocks, tabs, static_cast<double *>(U), Bi, grad);
  else k_ic<4, float><<<n, 256, 0, s>>>(blocks, tabs, static_cast<float *>(U), Bi, grad);
  return cudaGetLastError();
}

cudaError_t launch_refine(const Method &m, const TreeOpArgs &a, int n, cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  const int per = 4 * (m.ng == 2 ? refine_chunks<2>() : refine_chunks<4>());   // (son, chunk) CTAs per op
  AMR_DISPATCH_NG_S(m, k_refine, n * per, kRefineChunk, 0, s, a);
  return cudaGetLastError();
}

cudaError_t launch_coarsen(const Method &m, const TreeOpArgs &a, int n, cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  AMR_DISPATCH_NG_S(m, k_coarsen, n, 256, 0, s, a);
  return cudaGetLastError();
}

// Copy whole blocks between the slot pool and a dense float64 staging array
// (block b of the staging array <-> slot slots[b]), converting FP32 fields.
// blocks [0, nblk) of a field between the slot pool and a dense float64
// array [block][per] (device memory, or a host array the GPU addresses); two
// consecutive values per thread (`per` is even, so a pair never straddles
// blocks) when the dense array is 16-byte aligned
template <int W>
__global__ void k_gather(const int *slots, int nblk, const void *src, int f32, int per, double *dst) {
  const size_t total = static_cast<size_t>(nblk) * per / W;
  for (size_t e = blockIdx.x * static_cast<size_t>(blockDim.x) + threadIdx.x; e < total;
       e += static_cast<size_t>(gridDim.x) * blockDim.x) {
    const size_t i = e * W, b = i / per, r = i % per;
    const size_t s = static_cast<size_t>(slots[b]) * per + r;
    if (W == 2) {
      double2 v;
      if (f32) {
        const float2 f = *reinterpret_cast<const float2 *>(static_cast<const float *>(src) + s);
        v.x = f.x;
        v.y = f.y;
      } else {
        v = *reinterpret_cast<const double2 *>(static_cast<const double *>(src) + s);
      }
      *reinterpret_cast<double2 *>(dst + i) = v;
    } else {
      dst[i] = f32 ? static_cast<double>(static_cast<const float *>(src)[s]) : static_cast<const double *>(src)[s];
    }
  }
}

template <int W>
__global__ void k_scatter(const int *slots, int nblk, void *dst, int f32, int per, const double *src) {
  const size_t total = static_cast<size_t>(nblk) * per / W;
  for (size_t e = blockIdx.x * static_cast<size_t>(blockDim.x) + threadIdx.x; e < total;
       e += static_cast<size_t>(gridDim.x) * blockDim.x) {
    const size_t i = e * W, b = i / per, r = i % per;
    const size_t d = static_cast<size_t>(slots[b]) * per + r;
    if (W == 2) {
      const double2 v = *reinterpret_cast<const double2 *>(src + i);
      if (f32) *reinterpret_cast<float2 *>(static_cast<float *>(dst) + d) = make_float2(static_cast<float>(v.x),
                                                                                          static_cast<float>(v.y));
      else *reinterpret_cast<double2 *>(static_cast<double *>(dst) + d) = v;
    } else {
      if (f32) static_cast<float *>(dst)[d] = static_cast<float>(src[i]);
      else static_cast<double *>(dst)[d] = src[i];
    }
  }
}

namespace {
bool pairs_ok(const void *dense, int per) { return per % 2 == 0 && reinterpret_cast<uintptr_t>(dense) % 16 == 0; }
int xfer_grid(size_t items) { return static_cast<int>((items + 255) / 256 < 152 * 16 ? (items + 255) / 256 : 152 * 16); }
}  // namespace

cudaError_t launch_gather(const int *slots, int nblk, const void *src, int f32, int per, double *dst,
                          cudaStream_t s) {
  if (nblk <= 0) return cudaSuccess;
  const size_t total = static_cast<size_t>(nblk) * per;
  if (pairs_ok(dst, per)) k_gather<2><<<xfer_grid(total / 2), 256, 0, s>>>(slots, nblk, src, f32, per, dst);
  else k_gather<1><<<xfer_grid(total), 256, 0, s>>>(slots, nblk, src, f32, per, dst);
  return cudaGetLastError();
}

cudaError_t launch_scatter(const int *slots, int nblk, void *dst, int f32, int per, const double *src,
                           cudaStream_t s) {
  if (nblk <= 0) return cudaSuccess;
  const size_t total = static_cast<size_t>(nblk) * per;
  if (pairs_ok(src, per)) k_scatter<2><<<xfer_grid(total / 2), 256, 0, s>>>(slots, nblk, dst, f32, per, src);
  else k_scatter<1><<<xfer_grid(total), 256, 0, s>>>(slots, nblk, dst, f32, per, src);
  return cudaGetLastError();
}

}  // namespace amr
