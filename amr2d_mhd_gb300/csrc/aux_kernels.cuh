// Ghost-fill gathers, constrained transport, the CFL / refinement reduction
// and the prolongation / restriction kernels.
#pragma once

#include <type_traits>

#include "amr_common.h"
#include "ic.hpp"
#include "physics.cuh"
#include "stage.cuh"

namespace amr {

// ------------------------------------------------------------ ghost fills
// (GhostLaunch and the gather of one op: ghost.cuh)

// save the pre-fill values the same fill overwrites
template <int N>
__global__ void k_ghost_snap(GhostLaunch g) {
  pdl_wait();
  constexpr int NN = N * N;
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= g.nsnaps) return;
  const GhostSnap sn = g.snaps[r];
  if (sn.slot < 0) return;  // padding of an instance's range
  int q, k;
  const GhostSeg s = ghost_seg(g, blockIdx.y, q, k);
  const size_t at = (static_cast<size_t>(sn.slot) * s.nv + k) * NN + sn.pos;
  g.snapbuf[(static_cast<size_t>(q) * g.nsnaps + r) * 8 + k] =
      s.f32 ? static_cast<double>(static_cast<const float *>(s.field)[at]) : static_cast<const double *>(s.field)[at];
}

template <int N>
__global__ void k_ghost_apply(GhostLaunch g) {
  pdl_wait();
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= g.nops) return;
  const GhostOp op = g.ops[r];
  if (op.type == GOP_NOP) return;  // padding of an instance's range
  int q, k;
  const GhostSeg s = ghost_seg(g, blockIdx.y, q, k);
  const double *snap = g.snapbuf + static_cast<size_t>(q) * g.nsnaps * 8;
  if (s.f32) ghost_apply_one<N, float>(s, op, k, snap);
  else ghost_apply_one<N, double>(s, op, k, snap);
}

// ------------------------------------------------------------- CT2D.cpp
struct CtArgs {
  const LeafTask *tasks;
  const InstParams *inst;
  const void *ff, *gg;    // fluxes (storage type S)
  double *EMF;
  const double *Bsrc;     // CT2D's Bi argument
  double *Bnew;           // CT2D's Binew argument
  void *q;                // cell state corrected by the face average
  DevError *err;
  int step;
  int ntasks;             // leaf tasks (k_ct_coop)
  FillFuse fuse;          // fused fills: the consumed fill first, the next one's snapshots last
};

// prologue and epilogue of a per-block kernel of the step with fused fills
template <int N>
__device__ __forceinline__ void fuse_apply(const FillFuse &f, const LeafTask &t) {
  if (f.apply.nseg) {
    fill_apply_task<N, double>(f, t, threadIdx.x, blockDim.x, nullptr);
    __syncthreads();
  }
}
template <int N>
__device__ __forceinline__ void fuse_save(const FillFuse &f, const LeafTask &t) {
  if (f.save.nseg) {
    __syncthreads();
    fill_save_task<N>(f, t, threadIdx.x, blockDim.x);
  }
}

// CT2D.cpp:28-75, CTtype 2 ("upwind (not ready)", defs.hpp:34), for the block
// of task t: pressure and speed of every cell of q in shared memory (:36-40),
// then the corner EMF weighting the two flux averages by psi, which stays 1/2
// unless the corner sits at a strong pressure jump (beta = 0.5) in a strongly
// compressive flow (delta = 0.1).  Two terms of the divergence divide rho*v
// by itself (:52), as the reference does.  Arithmetic in the storage type S
// (FP64 on the FP64 path, in the reference's order).
template <int NG, typename S>
__device__ __forceinline__ void ct_emf_upwind(const CtArgs &a, const LeafTask &t, S *sp, S *sC) {
  constexpr int N = Geo<NG>::N, NN = N * N;
  const S g = static_cast<S>(a.inst[t.inst].gamma);
  const S *q = static_cast<const S *>(a.q) + static_cast<size_t>(t.slot) * 8 * NN;
  const S *ff = static_cast<const S *>(a.ff) + static_cast<size_t>(t.slot) * 8 * NN;
  const S *gg = static_cast<const S *>(a.gg) + static_cast<size_t>(t.slot) * 8 * NN;
  double *E = a.EMF + static_cast<size_t>(t.slot) * NN;
  for (int c = threadIdx.x; c < NN; c += blockDim.x) {
    const S q0 = q[c], q1 = q[NN + c], q2 = q[2 * NN + c], q3 = q[3 * NN + c];
    const S q4 = q[4 * NN + c], q5 = q[5 * NN + c], q6 = q[6 * NN + c], q7 = q[7 * NN + c];
    sp[c] = (g - S(1)) * (q4 - S(0.5) * ((q1 * q1 + q2 * q2 + q3 * q3) / q0 + (q5 * q5 + q6 * q6 + q7 * q7)));
    sC[c] = sqrt((g * sp[c] + (q5 * q5 + q6 * q6 + q7 * q7)) / q0);
  }
  __syncthreads();
  for (int c = threadIdx.x; c < NN; c += blockDim.x) {
    const int i = c % N, j = c / N;
    if (i < 1 || j < 1) continue;
    const int w = c - 1, s = c - N, sw = c - N - 1;  // (i-1,j), (i,j-1), (i-1,j-1)
    const S beta = S(0.5), delta = S(0.1);
    const S dPx = S(0.5) * fabs(sp[c] + sp[s] - sp[w] - sp[sw]);
    const S dPy = S(0.5) * fabs(sp[c] + sp[w] - sp[s] - sp[sw]);
    const S divV = S(0.5) * (q[NN + c] / q[c] + q[NN + s] / q[s] - q[NN + w] / q[w] - q[NN + sw] / q[sw]) +
                   S(0.5) * (q[2 * NN + c] / q[c] + q[2 * NN + w] / q[2 * NN + w] - q[2 * NN + s] / q[2 * NN + s] -
                             q[2 * NN + sw] / q[sw]);
    S tempP = mmin(sp[sw], sp[s]);
    const S tempP1 = mmin(sp[w], sp[c]);
    tempP = mmin(tempP, tempP1);
    const bool sw1 = (dPx + dPy) > beta * tempP;
    S tempC = mmin(sC[sw], sC[s]);
    const S tempC1 = mmin(sC[w], sC[c]);
    tempC = mmin(tempC, tempC1);
    const bool sw2 = (-delta * tempC) > divV;
    S psi = S(0.5);
    if (sw1 && sw2) psi = dPx / (dPx + dPy);
    if (psi < S(0) || psi > S(1)) dev_fail(a.err, DERR_PSI, t.slot, i, j, static_cast<double>(psi));
    E[c] = static_cast<double>(S(0.5) * (S(1.) - psi) * (gg[5 * NN + c - 1] + gg[5 * NN + c]) -
                               S(0.5) * psi * (ff[6 * NN + c - N] + ff[6 * NN + c]));
  }
}

// CT2D.cpp:16-26 corner EMF for i, j in [1, N), block of task t (sp, sC:
// shared scratch of the upwind form)
template <int NG, typename S>
__device__ __forceinline__ void ct_emf_block(const CtArgs &a, const FillFuse &f, const LeafTask &t, S *sp, S *sC) {
  constexpr int N = Geo<NG>::N, NN = N * N;
  fuse_apply<N>(f, t);
  if (a.inst[t.inst].ct_type == 2) {
    ct_emf_upwind<NG, S>(a, t, sp, sC);
    fuse_save<N>(f, t);
    return;
  }
  const S *ff = static_cast<const S *>(a.ff) + static_cast<size_t>(t.slot) * 8 * NN;
  const S *gg = static_cast<const S *>(a.gg) + static_cast<size_t>(t.slot) * 8 * NN;
  double *E = a.EMF + static_cast<size_t>(t.slot) * NN;
  for (int c = threadIdx.x; c < NN; c += blockDim.x) {
    const int i = c % N, j = c / N;
    if (i < 1 || j < 1) continue;
    // in the storage type of the fluxes: FP64 on the FP64 path (the
    // reference's arithmetic); FP32 fluxes give an FP32 EMF, stored in the
    // FP64 array (the face update below stays FP64, so div B keeps FP64
    // round-off whatever the EMF's precision)
    const S g5a = gg[5 * NN + j * N + i - 1], g5b = gg[5 * NN + c];
    const S f6a = ff[6 * NN + (j - 1) * N + i], f6b = ff[6 * NN + c];
    E[c] = static_cast<double>(S(0.25) * ((g5a + g5b) - (f6a + f6b)));
  }
  fuse_save<N>(f, t);
}

// CT2D.cpp:78-92 face update with the RK2 combine
template <int NG>
__device__ __forceinline__ void ct_face_block(const CtArgs &a, const FillFuse &f, const LeafTask &t) {
  constexpr int N = Geo<NG>::N, NN = N * N;
  fuse_apply<N>(f, t);
  const double dt = a.inst[t.inst].dt;
  const double *E = a.EMF + static_cast<size_t>(t.slot) * NN;
  const double *B0 = a.Bsrc + static_cast<size_t>(t.slot) * 2 * NN;
  double *B1 = a.Bnew + static_cast<size_t>(t.slot) * 2 * NN;
  for (int c = threadIdx.x; c < NN; c += blockDim.x) {
    const int i = c % N, j = c / N;
    const int ip = i < N - 1 ? i + 1 : i, jp = j < N - 1 ? j + 1 : j;
    double res = t.rcp_dy * (E[jp * N + i] - E[c]);
    if (a.step == 1) B1[c] = B0[c] - dt * res;
    else B1[c] = 0.5 * (B0[c] + B1[c] - dt * res);
    res = -t.rcp_dx * (E[j * N + ip] - E[c]);
    if (a.step == 1) B1[NN + c] = B0[NN + c] - dt * res;
    else B1[NN + c] = 0.5 * (B0[NN + c] + B1[NN + c] - dt * res);
  }
  fuse_save<N>(f, t);
}

// CT2D.cpp:95-123 cell B := face average, with the energy correction, on
// every cell of the block (ghosts included)
template <int NG, typename S>
__device__ __forceinline__ void ct_cell_block(const CtArgs &a, const FillFuse &f, const LeafTask &t) {
  constexpr int N = Geo<NG>::N, NN = N * N;
  fuse_apply<N>(f, t);
  const double *B = a.Bnew + static_cast<size_t>(t.slot) * 2 * NN;
  S *q = static_cast<S *>(a.q) + static_cast<size_t>(t.slot) * 8 * NN;
  for (int c = threadIdx.x; c < NN; c += blockDim.x) {
    const int i = c % N, j = c / N;
    const int ip = i < N - 1 ? i + 1 : i, ii = ip - 1;
    const int jp = j < N - 1 ? j + 1 : j, jj = jp - 1;
    // face averages from the FP64 face field, rounded once to the storage
    // type; the energy correction in the storage type (FP64 on the FP64 path)
    const S bx = static_cast<S>(0.5 * (B[j * N + ip] + B[j * N + ii]));
    const S by = static_cast<S>(0.5 * (B[NN + jp * N + i] + B[NN + jj * N + i]));
    const S q5 = q[5 * NN + c], q6 = q[6 * NN + c];
    q[4 * NN + c] = q[4 * NN + c] + S(0.5) * ((bx * bx + by * by) - (q5 * q5 + q6 * q6));
    q[5 * NN + c] = bx;
    q[6 * NN + c] = by;
  }
  fuse_save<N>(f, t);
}

template <int NG, typename S>
__global__ void k_ct_emf(CtArgs a) {
  pdl_wait();
  constexpr int NN = Geo<NG>::NN;
  __shared__ S sp[NN], sC[NN];
  ct_emf_block<NG, S>(a, a.fuse, a.tasks[blockIdx.x], sp, sC);
}

template <int NG>
__global__ void k_ct_face(CtArgs a) {
  pdl_wait();
  ct_face_block<NG>(a, a.fuse, a.tasks[blockIdx.x]);
}

template <int NG, typename S>
__global__ void k_ct_cell(CtArgs a) {
  pdl_wait();
  ct_cell_block<NG, S>(a, a.fuse, a.tasks[blockIdx.x]);
}

// Barrier of all CTAs of a cooperative grid (all resident at once): the last
// CTA to arrive zeroes the count and advances the generation.  The wait is
// bounded; a CTA that gives up records DERR_TIMEOUT and the barrier returns
// false in every thread of that CTA.
constexpr long kGridSpinLimit = 1L << 24;   // x 64 ns sleeps: about a second
__device__ __forceinline__ bool grid_barrier(unsigned *bar, DevError *err) {
  __shared__ int ok;
  __syncthreads();
  if (threadIdx.x == 0) {
    volatile unsigned *gen = bar + 1;
    const unsigned g = *gen;
    __threadfence();
    int good = 1;
    if (atomicAdd(bar, 1u) == gridDim.x - 1) {
      bar[0] = 0;
      __threadfence();
      atomicAdd(bar + 1, 1u);
    } else {
      for (long it = 0; *gen == g; it++) {
        if (it > kGridSpinLimit) { good = 0; break; }
        __nanosleep(64);
      }
      if (!good) dev_fail(err, DERR_TIMEOUT, -1, static_cast<int>(blockIdx.x), 0, 0.0);
    }
    __threadfence();
    ok = good;
  }
  __syncthreads();
  return ok != 0;
}

// CT2D.cpp:11-124 of one RK stage as one cooperative launch: the EMF, the
// face update and the cell correction, each over every leaf (a CTA takes
// tasks blockIdx.x, + gridDim.x, ...), separated by grid barriers.  The two
// fills CT2D makes between them (boundaryec on the EMF, boundaryfc on the new
// face field) are fused: gathered by the phase that consumes them, their
// snapshots saved by the phase before.  The EMF phase also gathers the fill
// of the fluxes and face field that precedes CT2D (main.cpp:161-163), and
// the cell phase saves the snapshots of the cell fill that follows it.
template <int NG, typename S, int THREADS>
__global__ void __launch_bounds__(THREADS) k_ct_coop(CtArgs a, FillFuse f_emf, FillFuse f_face, FillFuse f_cell,
                                                     unsigned *bar) {
  pdl_wait();
  constexpr int NN = Geo<NG>::NN;
  __shared__ S sp[NN], sC[NN];
  for (int ti = blockIdx.x; ti < a.ntasks; ti += gridDim.x) {
    ct_emf_block<NG, S>(a, f_emf, a.tasks[ti], sp, sC);
    __syncthreads();  // the upwind form's shared scratch is reused by the next task
  }
  if (!grid_barrier(bar, a.err)) return;
  for (int ti = blockIdx.x; ti < a.ntasks; ti += gridDim.x) ct_face_block<NG>(a, f_face, a.tasks[ti]);
  if (!grid_barrier(bar, a.err)) return;
  for (int ti = blockIdx.x; ti < a.ntasks; ti += gridDim.x) ct_cell_block<NG, S>(a, f_cell, a.tasks[ti]);
}

// diffusivity.cpp:6-17 on the blocks flagged TASK_DIFFUSE (main.cpp:190-193:
// after stage 2, level >= maxlevs - 2): U += eta * (5-point Laplacian) over
// the interior, eta = 0.001 (defs.hpp:50).  The reference sweeps in place
// with i outer and j inner, so a cell sees the new (i-1, j) and (i, j-1) and
// the old (i+1, j) and (i, j+1): the CTA sweeps the anti-diagonals i + j of
// the block in shared memory, 8 variables x 16 cells per diagonal.
template <int NG, typename S>
__global__ void __launch_bounds__(128) k_diffuse(CtArgs a) {
  pdl_wait();
  constexpr int N = Geo<NG>::N, NN = N * N, I0 = NG;  // interior [nxmin, nxmax] = [NG, NG + NI - 1]
  const LeafTask t = a.tasks[blockIdx.x];
  if (!(t.flags & TASK_DIFFUSE)) return;
  __shared__ S u[8 * NN];
  S *q = static_cast<S *>(a.q) + static_cast<size_t>(t.slot) * 8 * NN;
  for (int e = threadIdx.x; e < 8 * NN; e += blockDim.x) u[e] = q[e];
  __syncthreads();
  const S eta = S(0.001);
  const int k = threadIdx.x / NI, m = threadIdx.x % NI;
  for (int d = 0; d <= 2 * (NI - 1); d++) {
    const int i0 = (d > NI - 1 ? d - (NI - 1) : 0) + m;
    if (i0 <= (d < NI - 1 ? d : NI - 1)) {
      S *c = u + k * NN + (I0 + d - i0) * N + (I0 + i0);
      *c = *c + eta * (c[1] + c[-1] + c[N] + c[-N] - S(4.) * *c);
    }
    __syncthreads();
  }
  for (int e = threadIdx.x; e < 8 * NI * NI; e += blockDim.x) {
    const int kk = e / (NI * NI), r = e % (NI * NI);
    const int at = kk * NN + (I0 + r / NI) * N + I0 + r % NI;
    q[at] = u[at];
  }
}

// --------------------------------------------- dt (main.cpp:209-230) and
// refinement criterion (criteria.cpp:6-44) of every leaf: one CTA per leaf.
// The CTA first converts the block's U to primitives in shared memory
// (U2W("main"), main.cpp:213, with its pressure trap on the interior and its
// NaN trap on every cell, as k_prim), then one thread per interior cell
// forms the wave speeds and the criterion from them (FP64 for the FP64 path;
// the FP32 path computes the cell values in FP32 and reduces them in FP64).
__device__ __forceinline__ double warp_max(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const double u = __shfl_xor_sync(0xffffffffu, v, o);
    v = v < u ? u : v;
  }
  return v;
}

// warp maximum in the storage type (the reduction above, before widening)
template <typename T>
__device__ __forceinline__ T warp_max_t(T v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const T u = __shfl_xor_sync(0xffffffffu, v, o);
    v = v < u ? u : v;
  }
  return v;
}

struct DtArgs {
  const LeafTask *tasks;
  const InstParams *inst;
  const void *U;    // conserved state after the step
  double *lambda;   // per task: max over cells of max(|rho| + c_f,x, |u| + c_f,y)
  double *grad;     // per task: max relative jump
  DevError *err;
  int want_grad;
  FillFuse fuse;    // fused fills: the fill of U after the step, gathered first
};

template <int NG, typename S>
__global__ void __launch_bounds__(256) k_dt_cell(DtArgs a) {
  pdl_wait();
  using G = Geo<NG>;
  using T = S;
  constexpr int N = G::N, NN = G::NN, LO = G::LO, HI = G::HI;
  static_assert(NI * NI == 256, "one thread per interior cell");
  __shared__ double red[2][8];
  __shared__ S sW[8 * NN];
  const LeafTask t = a.tasks[blockIdx.x];
  fuse_apply<N>(a.fuse, t);
  const S *U = static_cast<const S *>(a.U) + static_cast<size_t>(t.slot) * 8 * NN;
  for (int c = threadIdx.x; c < NN; c += blockDim.x) {
    S u[8], w[8];
#pragma unroll
    for (int k = 0; k < 8; k++) u[k] = U[k * NN + c];
    cons2prim_cell<S>(u, w, a.inst[t.inst].gamma);
#pragma unroll
    for (int k = 0; k < 8; k++) sW[k * NN + c] = w[k];
    const int i = c % N, j = c / N;
    if (w[4] <= S(0) && i > LO && i < HI + 1 && j > LO && j < HI + 1)
      dev_fail(a.err, DERR_PRESSURE, t.slot, i, j, static_cast<double>(w[4]));
    bool bad = false;
#pragma unroll
    for (int k = 0; k < 8; k++) bad |= isnan(w[k]);
    if (bad) dev_fail(a.err, DERR_NAN, t.slot, i, j, 0.0);
  }
  __syncthreads();
  const T g = static_cast<T>(a.inst[t.inst].gamma);
  const int i = NG + threadIdx.x % NI, j = NG + threadIdx.x / NI, c = j * N + i;
  const S *W = sW;
  T w[8];
#pragma unroll
  for (int k = 0; k < 8; k++) w[k] = W[k * NN + c];
  // wavespeeds (misc.cpp:71-79) for norm 5 and 6; ca and a are the same
  // values in both calls.  lambda1 takes |rho| (main.cpp:222), lambda2 |u|.
  const T ca = sqrt((w[5] * w[5] + w[6] * w[6] + w[7] * w[7]) / w[0]);
  const T as = sqrt(g * w[4] / w[0]);
  T cf[2];
#pragma unroll
  for (int q = 0; q < 2; q++) {
    const T can = sqrt((w[5 + q] * w[5 + q]) / w[0]);
    const T i0 = (ca * ca) + (as * as), i1 = (ca * ca) - (as * as);
    cf[q] = sqrt(T(0.5) * (i0 + sqrt(i1 * i1 + T(4.) * (as * as) * ((ca * ca) - (can * can)))));
  }
  // the maxima in the storage type, widened to FP64 once per warp: the
  // widening is exact and monotonic, so this equals the maximum of the
  // widened values (and keeps FP32 maxima off the FP64 pipe)
  T lamT = smax(fabs(w[0]) + cf[0], fabs(w[1]) + cf[1]);
  T grT = T(0.);
  if (a.want_grad) {
#pragma unroll
    for (int q = 0; q < 4; q++) {
      const int v = q == 0 ? 4 : (q == 1 ? 0 : q + 3);   // p, rho, Bx, By
      const S *x = W + v * NN + c;
      const T c0 = x[0];
      const T dm = mmax(static_cast<T>(EPS), fabs(c0));
      T d1 = fabs(x[1] - c0);
      T d2 = mmax(d1, fabs(x[-1] - c0));
      d1 = mmax(d2, fabs(x[N] - c0));
      d2 = mmax(d1, fabs(x[-N] - c0));
      grT = mmax(grT, d2 / dm);
    }
  }
  const double lam = static_cast<double>(warp_max_t(lamT));
  const double gr = static_cast<double>(warp_max_t(grT));
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  if (lane == 0) { red[0][wid] = lam; red[1][wid] = gr; }
  __syncthreads();
  if (threadIdx.x == 0) {
    double mm = red[0][0], gg = red[1][0];
    for (int q = 1; q < 8; q++) {
      mm = mm < red[0][q] ? red[0][q] : mm;
      gg = gg < red[1][q] ? red[1][q] : gg;
    }
    a.lambda[blockIdx.x] = mm;
    a.grad[blockIdx.x] = gg;
  }
}

// ------------------------------------------------- initial condition (amr_init)
// IC2Dtype.cpp:6-190 + W2U (meshblock.cpp:181-199) for one root block per CTA:
// the primitive state of every cell (ghosts included) into shared memory and
// the conserved state to the block's slot, the face field from the cell
// averages (IC2Dtype.cpp:172-189), and the block's refinement criterion
// (criteria.cpp:11-29) for amr_init's first admesh.  Constants and the 1-D
// profiles that need the C library (sin, exp, cos) come from the host
// (IcDev, ic_prepare); everything else is evaluated here in the host code's
// order, without FMA contraction, so the state is the host evaluation's.
template <int NG, typename S>
__global__ void __launch_bounds__(256) k_ic(const IcDev *blocks, const double *tabs, S *U, double *Bi, double *grad) {
  constexpr int N = Geo<NG>::N, NN = N * N;
  __shared__ double sW[8 * NN];
  __shared__ double red[8];
  const IcDev d = blocks[blockIdx.x];
  const double *t0 = d.tab >= 0 ? tabs + static_cast<size_t>(d.tab) * N : nullptr;
  S *u = U + static_cast<size_t>(d.slot) * 8 * NN;
  for (int c = threadIdx.x; c < NN; c += blockDim.x) {
    const int i = c % N, j = c / N;
    const double x = ((i + d.icoord_x - NG) + 0.5) * d.dx - d.shift_x;
    const double y = ((j + d.icoord_y - NG) + 0.5) * d.dy - d.shift_y;
    double w[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    if (d.ic <= IC_BWY1) {  // quadrants, IC2Dtype.cpp:114-168
      int k;
      if (x >= 0.5 && y >= 0.5) k = 0;
      else if (x < 0.5 && y >= 0.5) k = 1;
      else if (x < 0.5 && y < 0.5) k = 2;
      else k = 3;
      w[0] = d.c[k]; w[4] = d.c[4 + k]; w[5] = d.c[8 + k]; w[6] = d.c[12 + k];
    } else if (d.ic == IC_ROTOR) {  // IC2Dtype.cpp:90-113
      const double radius = sqrt((x - 0.5) * (x - 0.5) + (y - 0.5) * (y - 0.5));
      const double fr = (23. - 200. * radius) / 3.;
      w[4] = 0.5;
      w[5] = d.c[0];
      if (radius <= 0.1) {
        w[0] = 10.; w[1] = -(y - 0.5) / 0.1; w[2] = (x - 0.5) / 0.1;
      } else if (radius > 0.1 && radius < 0.115) {
        w[0] = (1 + 9. * fr); w[1] = (-(y - 0.5) * fr / 0.1); w[2] = (x - 0.5) * fr / 0.1;
      } else {
        w[0] = 1.;
      }
    } else if (d.ic == IC_OT) {
      const double sx = t0[i], s2x = t0[N + i], sy = t0[2 * N + j];
      w[0] = d.c[0]; w[4] = d.c[1];
      w[1] = -sy; w[2] = sx;
      w[5] = -sy / d.c[2]; w[6] = s2x / d.c[2];
    } else if (d.ic == IC_BLAST) {
      const double rr = sqrt((x - d.c[4]) * (x - d.c[4]) + (y - d.c[5]) * (y - d.c[5]));
      w[0] = 1.0; w[4] = rr < d.c[0] ? d.c[1] : 0.1;
      w[5] = d.c[2]; w[6] = d.c[3];
    } else if (d.ic == IC_KH) {
      const bool in = fabs(y - 0.5) <= 0.25;
      w[0] = in ? 2.0 : 1.0; w[1] = in ? 0.5 : -0.5; w[4] = 2.5;
      w[5] = d.c[0];
      w[2] = t0[i] * t0[N + j];
    }
#pragma unroll
    for (int k = 0; k < 8; k++) sW[k * NN + c] = w[k];
    // W2U (meshblock.cpp:181-199)
    const double g = d.gamma;
    const double e = (w[4] / (g - 1)) + 0.5 * w[0] * (w[1] * w[1] + w[2] * w[2] + w[3] * w[3]);
    const double q[8] = {w[0], w[1] * w[0], w[2] * w[0], w[3] * w[0],
                         e + 0.5 * (w[5] * w[5] + w[6] * w[6] + w[7] * w[7]), w[5], w[6], w[7]};
#pragma unroll
    for (int k = 0; k < 8; k++) u[k * NN + c] = static_cast<S>(q[k]);
  }
  __syncthreads();
  // IC2Dtype.cpp:172-189: Bx at i-1/2 from the two cell averages (the first
  // face takes the second's value), By likewise
  double *bx = Bi + static_cast<size_t>(d.slot) * 2 * NN, *by = bx + NN;
  for (int c = threadIdx.x; c < NN; c += blockDim.x) {
    const int i = c % N, j = c / N;
    const int il = i > 0 ? i - 1 : 0, jl = j > 0 ? j - 1 : 0;
    bx[c] = 0.5 * (sW[5 * NN + j * N + il] + sW[5 * NN + j * N + il + 1]);
    by[c] = 0.5 * (sW[6 * NN + jl * N + i] + sW[6 * NN + (jl + 1) * N + i]);
  }
  // criteria.cpp:11-29 over the interior (one thread per interior cell)
  static_assert(NI * NI == 256, "one thread per interior cell");
  const int i = NG + threadIdx.x % NI, j = NG + threadIdx.x / NI, c = j * N + i;
  double gr = 0;
#pragma unroll
  for (int q = 0; q < 4; q++) {
    const int v = q == 0 ? 4 : (q == 1 ? 0 : q + 3);   // p, rho, Bx, By
    const double *x = sW + v * NN + c;
    const double c0 = x[0];
    const double dm = 1.0E-15 > fabs(c0) ? 1.0E-15 : fabs(c0);
    double dd = fabs(x[1] - c0);
    double ee = fabs(x[-1] - c0);
    dd = dd > ee ? dd : ee;
    ee = fabs(x[N] - c0);
    dd = dd > ee ? dd : ee;
    ee = fabs(x[-N] - c0);
    dd = dd > ee ? dd : ee;
    const double r = dd / dm;
    gr = gr > r ? gr : r;
  }
  gr = warp_max(gr);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = gr;
  __syncthreads();
  if (threadIdx.x == 0) {
    double m = red[0];
    for (int q = 1; q < 8; q++) m = m < red[q] ? red[q] : m;
    grad[blockIdx.x] = m;
  }
}

// -------------------------------------------- refine.cpp / refineBi_CT.cpp
struct TreeOpArgs {
  const TreeOp *ops;
  const InstParams *inst;
  void *U;
  double *Bi;
  DevError *err;
};

// refine.cpp:17-85 (minmod, the slope multiplies the forward difference) and
// U2W("refine") on the sons, then refineBi_CT.cpp:4-74 for the face field.
// Work is spread over many CTAs: CTA (op, son, chunk) takes kRefineChunk
// cells of one son, one thread per cell (8 variables and 2 face components),
// so the FP64 divisions of a refined block run on many SMs at once.
constexpr int kRefineChunk = 128;
template <int NG> __host__ __device__ constexpr int refine_chunks() {
  return (Geo<NG>::NN + kRefineChunk - 1) / kRefineChunk;
}

template <int NG, typename S>
__global__ void __launch_bounds__(kRefineChunk) k_refine(TreeOpArgs a) {
  using G = Geo<NG>;
  constexpr int N = G::N, NN = G::NN, n2 = (N - 1) / 2, CH = refine_chunks<NG>();
  using T = S;
  const int opi = blockIdx.x / (4 * CH), sq = (blockIdx.x / CH) % 4;
  const int c = (blockIdx.x % CH) * kRefineChunk + threadIdx.x;
  if (c >= NN) return;
  const TreeOp op = a.ops[opi];
  const S *D = static_cast<const S *>(a.U) + static_cast<size_t>(op.dad) * 8 * NN;
  const T E = eps_of<T>();
  // refine.cpp:45-59 for cell c of son sq, its 8 variables
  {
    const int i = c % N, j = c / N;
    const int sx = (i + NG) % 2, sy = (j + NG) % 2;
    const int ii = (sq & 1) ? (i - NG + 2) / 2 + n2 : (i + NG) / 2;
    const int jj = (sq & 2) ? (j - NG + 2) / 2 + n2 : (j + NG) / 2;
    S *Sn = static_cast<S *>(a.U) + static_cast<size_t>(op.son[sq]) * 8 * NN;
    T u[8];
#pragma unroll
    for (int k = 0; k < 8; k++) {
      const S *q = D + k * NN;
      const T q0 = q[jj * N + ii];
      T res = q0, r, phi;
      r = (q0 - q[jj * N + ii - 1]) / (q[jj * N + ii + 1] - q0 + E);
      phi = T(0.25) * slope_limiter<T>(LIM_MINMOD, r, T(0)) * (q[jj * N + ii + 1] - q0);
      res = sx == 0 ? res - phi : res + phi;
      r = (q0 - q[(jj - 1) * N + ii]) / (q[(jj + 1) * N + ii] - q0 + E);
      phi = T(0.25) * slope_limiter<T>(LIM_MINMOD, r, T(0)) * (q[(jj + 1) * N + ii] - q0);
      res = sy == 0 ? res - phi : res + phi;
      u[k] = res;
      Sn[k * NN + c] = res;
    }
    // U2W("refine") pressure trap (refine.cpp:70-82)
    T w[8];
    cons2prim_cell<S>(u, w, a.inst[op.inst].gamma);
    if (w[4] <= T(0) && i > G::LO && i < G::HI + 1 && j > G::LO && j < G::HI + 1)
      dev_fail(a.err, DERR_PRESSURE, op.son[sq], i, j, static_cast<double>(w[4]));
  }
  // refineBi_CT.cpp:4-74, both face components of cell c of son sq
  const double *Bd = a.Bi + static_cast<size_t>(op.dad) * 2 * NN;
  const int i0 = c % N, j0 = c / N;
  const int sx = (i0 + NG) % 2, sy = (j0 + NG) % 2;
  const int i = (sq & 1) ? (i0 - NG + 2) / 2 + n2 : (i0 + NG) / 2;
  const int j = (sq & 2) ? (j0 - NG + 2) / 2 + n2 : (j0 + NG) / 2;
  const double *bx = Bd, *by = Bd + NN;
  auto X = [&](int di, int dj) { return bx[(j + dj) * N + i + di]; };
  auto Y = [&](int di, int dj) { return by[(j + dj) * N + i + di]; };
  const double Bx_jm = X(0, -1), Bx = X(0, 0), Bx_jp = X(0, 1);
  const double Bx_ip = X(1, 0), Bx_ipjm = X(1, -1), Bx_ipjp = X(1, 1);
  const double By_im = Y(-1, 0), By = Y(0, 0), By_ip = Y(1, 0);
  const double By_imjp = Y(-1, 1), By_jp = Y(0, 1), By_ipjp = Y(1, 1);
  double r;
  r = (Bx - Bx_jm) / (Bx_jp - Bx + EPS);
  const double DyBxm = slope_limiter<double>(LIM_MINMOD, r, 0) * (Bx_jp - Bx);
  r = (Bx_ip - Bx_ipjm) / (Bx_ipjp - Bx_ip + EPS);
  const double DyBxp = slope_limiter<double>(LIM_MINMOD, r, 0) * (Bx_ipjp - Bx_ip);
  r = (By - By_im) / (By_ip - By + EPS);
  const double DxBym = slope_limiter<double>(LIM_MINMOD, r, 0) * (By_ip - By);
  r = (By_jp - By_imjp) / (By_ipjp - By_jp + EPS);
  const double DxByp = slope_limiter<double>(LIM_MINMOD, r, 0) * (By_ipjp - By_jp);
  const double ax = (Bx_ip - Bx);
  const double by_ = -1. * ax;
  const double ay = 0.5 * (DyBxp + DyBxm);
  const double bx_ = 0.5 * (DxByp + DxBym);
  const double axy = (DyBxp - DyBxm);
  const double byy = axy / (-2.);
  const double bxy = (DxByp - DxBym);
  const double axx = bxy / (-2.);
  const double a0 = 0.5 * (Bx_ip + Bx) - 0.25 * axx;
  const double b0 = 0.5 * (By_jp + By) - 0.25 * byy;
  const double ayy = 0., bxx = 0.;
  double *out = a.Bi + static_cast<size_t>(op.son[sq]) * 2 * NN + c;
#pragma unroll
  for (int k = 0; k < 2; k++) {
    double res;
    if (k == 0) {
      const double tx = sx == 0 ? 0 : 0.5, ty = sy == 0 ? -0.25 : 0.25;
      res = a0 + ax * tx + ay * ty + axx * tx * tx + axy * tx * ty + ayy * ty * ty;
    } else {
      const double tx = sx == 0 ? -0.25 : 0.25, ty = sy == 0 ? 0 : 0.5;
      res = b0 + bx_ * tx + by_ * ty + bxx * tx * tx + bxy * tx * ty + byy * ty * ty;
    }
    if (isnan(res)) dev_fail(a.err, DERR_REFINE_NAN, op.son[sq], i0, j0, 0.0);
    out[k * NN] = res;
  }
}

// ------------------------------------------- coarsen.cpp / coarsenBi_CT.cpp
// The reference's nine loop nests run in order (a cell written by two nests
// keeps the later value); each nest is spread over the CTA.
template <int NG, typename F, bool FACE>
__device__ void coarsen_field(F *Q, int nv, const int *son, int dad) {
  using G = Geo<NG>;
  constexpr int N = G::N, NN = G::NN, ng = NG;
  constexpr int nxmin = NG, nymin = NG, nxminb = NG - 1, nyminb = NG - 1;
  constexpr int nxmaxb = G::HI + 1, nymaxb = G::HI + 1, nx2 = (N - 1) / 2, ny2 = (N - 1) / 2;
  const F c = FACE ? F(0.5) : F(0.25);
  auto SUM = [&](int sb, int k, int i1, int j1) -> F {
    const F *s = Q + (static_cast<size_t>(sb) * nv + k) * NN;
    const int i2 = FACE ? (k == 0 ? i1 : i1 + 1) : i1 + 1;
    const int j2 = FACE ? (k == 0 ? j1 + 1 : j1) : j1 + 1;
    F v = F(0.);
    for (int i = i1; i <= i2; i++)
      for (int j = j1; j <= j2; j++) v += s[j * N + i];
    return c * v;
  };
  auto D = [&](int k, int i, int j) -> F & { return Q[(static_cast<size_t>(dad) * nv + k) * NN + j * N + i]; };
  const int tid = threadIdx.x, nt = blockDim.x;
  // the block itself
  {
    constexpr int ni = nx2 - nxmin + 1;
    for (int e = tid; e < ni * ni * nv; e += nt) {
      const int k = e / (ni * ni), r = e % (ni * ni);
      const int i = nxmin + r % ni, j = nymin + r / ni;
      const int i1 = 2 * i - nxmin, j1 = 2 * j - nymin;
      const int nx2i = nx2 + i - 1 - (ng - 2), ny2j = ny2 + j - 1 - (ng - 2);
      D(k, i, j) = SUM(son[0], k, i1, j1);
      D(k, nx2i, j) = SUM(son[1], k, i1, j1);
      D(k, i, ny2j) = SUM(son[2], k, i1, j1);
      D(k, nx2i, ny2j) = SUM(son[3], k, i1, j1);
    }
  }
  __syncthreads();
  constexpr int h = ng / 2;
  constexpr int nj = ny2 - nymin + 1;
  // Left corners
  for (int e = tid; e < nv * h * h; e += nt) {
    const int k = e / (h * h), i = (e % (h * h)) / h, j = e % h;
    const int i1 = nxminb - 2 * i - 1;
    int j1 = nyminb - 2 * j - 1;
    D(k, nxminb - i, nyminb - j) = SUM(son[0], k, i1, j1);
    j1 = nymaxb + 2 * j;
    D(k, nxminb - i, nymaxb + j) = SUM(son[2], k, i1, j1);
  }
  __syncthreads();
  // Left edge
  for (int e = tid; e < (nxminb + 1) * nj * nv; e += nt) {
    const int k = e / ((nxminb + 1) * nj), r = e % ((nxminb + 1) * nj);
    const int i = r / nj, j = nymin + r % nj;
    const int j1 = 2 * j - nymin, ny2j = j + ny2 - 1 - (ng - 2);
    int i1 = nxminb - 2 * i - 1;
    if (i1 < 0) i1 = 0;
    D(k, nxminb - i, j) = SUM(son[0], k, i1, j1);
    D(k, nxminb - i, ny2j) = SUM(son[2], k, i1, j1);
  }
  __syncthreads();
  // Right corners
  for (int e = tid; e < nv * h * h; e += nt) {
    const int k = e / (h * h), i = (e % (h * h)) / h, j = e % h;
    const int i1 = nxmaxb + 2 * i;
    int j1 = nyminb - 2 * j - 1;
    D(k, nxmaxb + i, nyminb - j) = SUM(son[1], k, i1, j1);
    j1 = nymaxb + 2 * j;
    D(k, nxmaxb + i, nymaxb + j) = SUM(son[3], k, i1, j1);
  }
  __syncthreads();
  // Right edge
  for (int e = tid; e < ng * nj * nv; e += nt) {
    const int k = e / (ng * nj), r = e % (ng * nj);
    const int i = r / nj, j = nymin + r % nj;
    const int j1 = 2 * j - nymin, ny2j = j + ny2 - 1 - (ng - 2);
    int i1 = nxmaxb + 2 * i;
    if (i1 + 1 > N - 1) i1 = N - 2;
    D(k, nxmaxb + i, j) = SUM(son[1], k, i1, j1);
    D(k, nxmaxb + i, ny2j) = SUM(son[3], k, i1, j1);
  }
  __syncthreads();
  // Bottom corners
  for (int e = tid; e < nv * h * h; e += nt) {
    const int k = e / (h * h), j = (e % (h * h)) / h, i = e % h;
    const int j1 = nyminb - 2 * j - 1;
    int i1 = nxminb - 2 * i - 1;
    D(k, nxminb - i, nyminb - j) = SUM(son[0], k, i1, j1);
    i1 = nxmaxb + 2 * i;
    D(k, nxmaxb + i, nyminb - j) = SUM(son[1], k, i1, j1);
  }
  __syncthreads();
  // Bottom edge
  for (int e = tid; e < nj * (nyminb + 1) * nv; e += nt) {
    const int k = e / (nj * (nyminb + 1)), r = e % (nj * (nyminb + 1));
    const int i = nxmin + r / (nyminb + 1), j = r % (nyminb + 1);
    const int i1 = 2 * i - nxmin, nx2i = i + nx2 - 1 - (ng - 2);
    int j1 = nyminb - 2 * j - 1;
    if (j1 < 0) j1 = 0;
    D(k, i, nyminb - j) = SUM(son[0], k, i1, j1);
    D(k, nx2i, nyminb - j) = SUM(son[1], k, i1, j1);
  }
  __syncthreads();
  // Top corners
  for (int e = tid; e < nv * h * h; e += nt) {
    const int k = e / (h * h), j = (e % (h * h)) / h, i = e % h;
    const int j1 = nymaxb + 2 * j;
    int i1 = nxminb - 2 * i - 1;
    D(k, nxminb - i, nymaxb + j) = SUM(son[2], k, i1, j1);
    i1 = nxmaxb + 2 * i;
    D(k, nxmaxb + i, nymaxb + j) = SUM(son[3], k, i1, j1);
  }
  __syncthreads();
  // Top edge
  for (int e = tid; e < nj * ng * nv; e += nt) {
    const int k = e / (nj * ng), r = e % (nj * ng);
    const int i = nxmin + r / ng, j = r % ng;
    const int i1 = 2 * i - nxmin, nx2i = i + nx2 - 1 - (ng - 2);
    int j1 = nymaxb + 2 * j;
    if (j1 + 1 > N - 1) j1 = N - 2;
    D(k, i, nymaxb + j) = SUM(son[2], k, i1, j1);
    D(k, nx2i, nymaxb + j) = SUM(son[3], k, i1, j1);
  }
  __syncthreads();
}

template <int NG, typename S>
__global__ void k_coarsen(TreeOpArgs a) {
  using G = Geo<NG>;
  constexpr int N = G::N, NN = G::NN;
  const TreeOp op = a.ops[blockIdx.x];
  coarsen_field<NG, S, false>(static_cast<S *>(a.U), 8, op.son, op.dad);
  // coarsen.cpp:151 U2W("coarsen") pressure trap on the dad
  const S *D = static_cast<const S *>(a.U) + static_cast<size_t>(op.dad) * 8 * NN;
  for (int c = threadIdx.x; c < NN; c += blockDim.x) {
    S u[8], w[8];
#pragma unroll
    for (int k = 0; k < 8; k++) u[k] = D[k * NN + c];
    cons2prim_cell<S>(u, w, a.inst[op.inst].gamma);
    const int i = c % N, j = c / N;
    if (w[4] <= S(0) && i > G::LO && i < G::HI + 1 && j > G::LO && j < G::HI + 1)
      dev_fail(a.err, DERR_PRESSURE, op.dad, i, j, static_cast<double>(w[4]));
  }
  coarsen_field<NG, double, true>(a.Bi, 2, op.son, op.dad);
}

}  // namespace amr
