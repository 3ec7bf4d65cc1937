// The RK stage as three kernels: primitive variables, Riemann fluxes, and the
// residual + RK update.  Same arithmetic as the fused k_stage (stage.cuh); the
// face kernel spreads the FP64-bound flux work of all leaves evenly over the
// SMs (one thread per face) instead of one CTA per block, and the primitive
// state and fluxes travel through L2 (the whole working set of a step is well
// below the 129 MB L2).
#pragma once

#include "stage.cuh"

namespace amr {

struct SplitArgs {
  const LeafTask *tasks;
  const InstParams *inst;
  const void *qin;    // U (stage 1) or Us (stage 2)
  void *qout;         // Us (stage 1) or U (stage 2)
  void *W;            // primitive state pool [slot][8][N][N]
  const double *B;    // Bi (stage 1) or Bis (stage 2)
  void *ff;
  void *gg;
  DevError *err;
  unsigned *ctr;      // [2] work counter and finished-CTA counter of k_faces_dyn (zero between launches)
  int step;
  int ntasks;
  FillFuse fuse;      // fused fills: the qin fill gathered by k_prim_task, the
                      // flux fill's snapshots saved by k_resid
};

// U2W / Us2W (meshblock.cpp:119-179) for every cell of every leaf
template <int NG, typename S>
__global__ void __launch_bounds__(512) k_prim(SplitArgs a) {
  pdl_wait();
  using G = Geo<NG>;
  constexpr int N = G::N, NN = G::NN, LO = G::LO, HI = G::HI;
  const size_t e = static_cast<size_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (e >= static_cast<size_t>(a.ntasks) * NN) return;
  const int t = static_cast<int>(e / NN), c = static_cast<int>(e % NN);
  const LeafTask task = a.tasks[t];
  const size_t base = static_cast<size_t>(task.slot) * 8 * NN;
  const S *Q = static_cast<const S *>(a.qin) + base;
  S *W = static_cast<S *>(a.W) + base;
  S u[8], w[8];
#pragma unroll
  for (int k = 0; k < 8; k++) u[k] = Q[k * NN + c];
  cons2prim_cell<S>(u, w, a.inst[task.inst].gamma);
#pragma unroll
  for (int k = 0; k < 8; k++) W[k * NN + c] = w[k];
  const int i = c % N, j = c / N;
  if (w[4] <= S(0) && i > LO && i < HI + 1 && j > LO && j < HI + 1)
    dev_fail(a.err, DERR_PRESSURE, task.slot, i, j, static_cast<double>(w[4]));
  bool bad = false;
#pragma unroll
  for (int k = 0; k < 8; k++) bad |= bits_nan(w[k]);
  if (bad) dev_fail(a.err, DERR_NAN, task.slot, i, j, 0.0);
}

// the same with the fill of qin (and B) fused in: one CTA per leaf gathers
// its block's ghost cells, then converts the block
template <int NG, typename S>
__global__ void __launch_bounds__(256) k_prim_task(SplitArgs a) {
  pdl_wait();
  using G = Geo<NG>;
  constexpr int N = G::N, NN = G::NN, LO = G::LO, HI = G::HI;
  const LeafTask task = a.tasks[blockIdx.x];
  fill_apply_task<N, double>(a.fuse, task, threadIdx.x, blockDim.x, nullptr);
  __syncthreads();
  const size_t base = static_cast<size_t>(task.slot) * 8 * NN;
  const S *Q = static_cast<const S *>(a.qin) + base;
  S *W = static_cast<S *>(a.W) + base;
  const double gamma = a.inst[task.inst].gamma;
  for (int c = threadIdx.x; c < NN; c += blockDim.x) {
    S u[8], w[8];
#pragma unroll
    for (int k = 0; k < 8; k++) u[k] = Q[k * NN + c];
    cons2prim_cell<S>(u, w, gamma);
#pragma unroll
    for (int k = 0; k < 8; k++) W[k * NN + c] = w[k];
    const int i = c % N, j = c / N;
    if (w[4] <= S(0) && i > LO && i < HI + 1 && j > LO && j < HI + 1)
      dev_fail(a.err, DERR_PRESSURE, task.slot, i, j, static_cast<double>(w[4]));
    bool bad = false;
#pragma unroll
    for (int k = 0; k < 8; k++) bad |= bits_nan(w[k]);
    if (bad) dev_fail(a.err, DERR_NAN, task.slot, i, j, 0.0);
  }
}

// MUSCL2D.cpp:24-116 for one face of one leaf: x faces (i+1/2, j) for i, j in
// [LO, HI], then y faces (i, j+1/2)
template <int NG, int RECON, int FLUX, typename S>
__device__ __forceinline__ void face_flux(const SplitArgs &a, size_t e) {
  using G = Geo<NG>;
  using T = S;
  constexpr int N = G::N, NN = G::NN, LO = G::LO, NF = G::NF, PER = 2 * NF * NF;
  const int t = static_cast<int>(e / PER), f = static_cast<int>(e % PER);
  const LeafTask task = a.tasks[t];
  const InstParams ip = a.inst[task.inst];
  const size_t base = static_cast<size_t>(task.slot) * 8 * NN;
  const S *W = static_cast<const S *>(a.W) + base;
  const bool yf = f >= NF * NF;
  const int g = yf ? f - NF * NF : f;
  const int r = g / NF, c = g % NF;
  const int s = yf ? N : 1;
  const int cL = (LO + r) * N + (LO + c);
  const int kn = yf ? 6 : 5;
  const T gamma = static_cast<T>(ip.gamma);
  T wl[8], wr[8];
#pragma unroll
  for (int k = 0; k < 8; k++) {
    if (k == kn) continue;
    const S *w = W + k * NN + cL;
    if (RECON == REC_MUSCL) {
      const T wm = w[-s], w0 = w[0], w1 = w[s], w2 = w[2 * s];
      muscl_face<T>(ip.limiter, w0, w1, w0 - wm, w1 - w0, w2 - w1, static_cast<T>(yf ? task.dy : task.dx),
                    wl[k], wr[k]);
    } else if (RECON == REC_WENO3) {
      T dummy;
      weno3_cell<T>(w[-s], w[0], w[s], wl[k], dummy);
      weno3_cell<T>(w[0], w[s], w[2 * s], dummy, wr[k]);
    } else {
      wl[k] = weno5_cell<T, false>(w[-2 * s], w[-s], w[0], w[s], w[2 * s]);
      wr[k] = weno5_cell<T, true>(w[-s], w[0], w[s], w[2 * s], w[3 * s]);
    }
  }
  const int fpos = cL + s;
  const double *Bf = a.B + static_cast<size_t>(task.slot) * 2 * NN + (yf ? NN : 0);
  const T bn = static_cast<T>(Bf[fpos]);
  wl[kn] = bn;
  wr[kn] = bn;
  T fl[8];
  int rc;
  if (!yf) {
    rc = riemann<FLUX, T>(wl, wr, gamma, fl);
  } else {
    T l2[8], r2[8], f2[8];
#pragma unroll
    for (int k = 0; k < 8; k++) { l2[k] = wl[k]; r2[k] = wr[k]; }
    l2[1] = wl[2]; l2[2] = wl[1]; r2[1] = wr[2]; r2[2] = wr[1];
    l2[5] = wl[6]; l2[6] = wl[5]; r2[5] = wr[6]; r2[6] = wr[5];
    rc = riemann<FLUX, T>(l2, r2, gamma, f2);
#pragma unroll
    for (int k = 0; k < 8; k++) fl[k] = f2[k];
    fl[1] = f2[2]; fl[2] = f2[1]; fl[5] = f2[6]; fl[6] = f2[5];
  }
  if (rc) dev_fail(a.err, rc, task.slot, fpos % N, fpos / N, 0.0);
  S *out = static_cast<S *>(yf ? a.gg : a.ff) + base + fpos;
  bool bad = false;
#pragma unroll
  for (int k = 0; k < 8; k++) {
    bad |= bits_nan(fl[k]);
    out[k * NN] = fl[k];
  }
  if (bad) dev_fail(a.err, DERR_NAN, task.slot, fpos % N, fpos / N, 0.0);
}

template <int NG, int RECON, int FLUX, typename S, int MINB>
__global__ void __launch_bounds__(128, MINB) k_faces(SplitArgs a) {
  pdl_wait();
  constexpr int PER = 2 * Geo<NG>::NF * Geo<NG>::NF;
  const size_t e = static_cast<size_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (e >= static_cast<size_t>(a.ntasks) * PER) return;
  face_flux<NG, RECON, FLUX, S>(a, e);
}

// persistent variant: a grid sized to the CTAs the SMs hold at once walks
// the whole face list of the step (all leaf blocks of all instances)
template <int NG, int RECON, int FLUX, typename S, int MINB>
__global__ void __launch_bounds__(128, MINB) k_faces_persist(SplitArgs a) {
  pdl_wait();
  constexpr int PER = 2 * Geo<NG>::NF * Geo<NG>::NF;
  const size_t n = static_cast<size_t>(a.ntasks) * PER;
  const size_t stride = static_cast<size_t>(gridDim.x) * blockDim.x;
  for (size_t e = static_cast<size_t>(blockIdx.x) * blockDim.x + threadIdx.x; e < n; e += stride)
    face_flux<NG, RECON, FLUX, S>(a, e);
}

// persistent variant with dynamic work distribution: a grid of the CTAs the
// SMs hold at once, each warp claiming the next 32 faces of the step's face
// list from a global counter, so that warps that met cheap faces (uniform
// regions, where the limiter ratios need no division) take more; the last
// CTA to finish zeroes the counters for the next launch (every CTA has left
// its loop by then, so nothing claims work any more)
template <int NG, int RECON, int FLUX, typename S, int MINB>
__global__ void __launch_bounds__(128, MINB) k_faces_dyn(SplitArgs a) {
  pdl_wait();
  constexpr int PER = 2 * Geo<NG>::NF * Geo<NG>::NF;
  const unsigned n = static_cast<unsigned>(a.ntasks) * PER;
  const int lane = threadIdx.x & 31;
  for (;;) {
    unsigned base = 0;
    if (lane == 0) base = atomicAdd(&a.ctr[0], 32u);
    base = __shfl_sync(0xffffffffu, base, 0);
    if (base >= n) break;
    if (base + lane < n) face_flux<NG, RECON, FLUX, S>(a, base + lane);
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    __threadfence();
    if (atomicAdd(&a.ctr[1], 1u) == gridDim.x - 1) {
      a.ctr[0] = 0;
      a.ctr[1] = 0;
    }
  }
}

// residual on [LO, HI]^2 (zero elsewhere) and the RK stage on every cell
// (main.cpp:147-157 / 179-189)
template <int NG, typename S>
__global__ void __launch_bounds__(512) k_resid(SplitArgs a) {
  pdl_wait();
  using G = Geo<NG>;
  using T = S;
  constexpr int N = G::N, NN = G::NN, LO = G::LO, HI = G::HI;
  const size_t e = static_cast<size_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  // fused fill: the flux fill's snapshots (this kernel writes only qout)
  if (a.fuse.save.nseg) fill_save_all<N>(a.fuse, e, static_cast<size_t>(gridDim.x) * blockDim.x);
  if (e >= static_cast<size_t>(a.ntasks) * 8 * NN) return;
  const int t = static_cast<int>(e / (8 * NN)), r = static_cast<int>(e % (8 * NN));
  const int c = r % NN;
  const int i = c % N, j = c / N;
  const LeafTask task = a.tasks[t];
  const size_t idx = static_cast<size_t>(task.slot) * 8 * NN + r;
  T res = T(0.);
  if (i >= LO && i <= HI && j >= LO && j <= HI) {
    const S *ff = static_cast<const S *>(a.ff) + idx;
    const S *gg = static_cast<const S *>(a.gg) + idx;
    if (task.inv_dx != 0.0 && task.inv_dy != 0.0)  // power-of-two cells: exact reciprocal
      res = (ff[1] - ff[0]) * static_cast<T>(task.inv_dx) + (gg[N] - gg[0]) * static_cast<T>(task.inv_dy);
    else
      res = (ff[1] - ff[0]) / static_cast<T>(task.dx) + (gg[N] - gg[0]) / static_cast<T>(task.dy);
  }
  const T dt = static_cast<T>(a.inst[task.inst].dt);
  const T q = static_cast<const S *>(a.qin)[idx];
  S *out = static_cast<S *>(a.qout) + idx;
  if (a.step == 1) *out = q - dt * res;
  else *out = T(0.5) * (*out + q - dt * res);
}

}  // namespace amr
