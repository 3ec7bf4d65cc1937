// Discrete adjoint of one fixed-mesh time step: MUSCL reconstruction with the
// MC / minmod limiter, the Rusanov flux, the residual and RK2 combine, CT2D and
// the ghost fills.  Every kernel is the transpose of the forward kernel of the
// same name (stage_split.cuh, aux_kernels.cuh) at the forward state it is
// given; FP64 only.  An adjoint array holds d(loss)/d(value) of the forward
// array of the same layout ([slot][var][N][N]).
#pragma once

#include "amr_common.h"
#include "aux_kernels.cuh"
#include "physics.cuh"
#include "stage.cuh"

namespace amr {

// ------------------------------------------------------------ ghost fills
// A fill writes dst <- f(pre-fill sources).  Its transpose moves the adjoint
// of every written cell to the cells it was read from: first take (read and
// zero) the adjoint of every destination, then add it to the sources.
struct GhostAdjLaunch {
  const GhostOp *ops;
  const GhostSnap *snaps;
  int nops;
  GhostSeg seg[kMaxSeg];   // adjoint arrays (double), nv and kind of the forward field
  int nseg;
  double *take;            // [nseg][nops][16]: per variable, the op's cell (and its pair)
};

template <int N>
__global__ void k_ghost_adj_take(GhostAdjLaunch g) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= g.nops * g.nseg) return;
  const int q = t / g.nops, r = t % g.nops;
  const GhostOp op = g.ops[r];
  if (op.type == GOP_NOP) return;
  const GhostSeg &s = g.seg[q];
  double *a = static_cast<double *>(s.field) + static_cast<size_t>(op.dst_slot) * s.nv * (N * N) + op.dst_pos;
  double *out = g.take + (static_cast<size_t>(q) * g.nops + r) * 16;
  for (int k = 0; k < s.nv; k++) {
    out[k] = a[k * N * N];
    a[k * N * N] = 0.0;
    if (op.type == GOP_COPY2) {  // the pair's second cell
      out[8 + k] = a[k * N * N + 1];
      a[k * N * N + 1] = 0.0;
    }
  }
}

// weights of the 2x2 patch (i,j) (i,j+1) (i+1,j) (i+1,j+1) in fine_value()
__device__ __forceinline__ void fine_weights(int kind, int k, double w[4]) {
  if (kind == 0) { w[0] = w[1] = w[2] = w[3] = 0.25; return; }
  w[0] = w[1] = w[2] = w[3] = 0.0;
  if (kind == 1) { w[0] = 0.5; if (k == 0) w[1] = 0.5; else w[2] = 0.5; return; }
  w[0] = 1.0;
}

template <int N>
__global__ void k_ghost_adj_give(GhostAdjLaunch g) {
  constexpr int NN = N * N;
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= g.nops * g.nseg) return;
  const int q = t / g.nops, r = t % g.nops;
  const GhostOp op = g.ops[r];
  if (op.type == GOP_NOP) return;
  const GhostSeg &s = g.seg[q];
  double *fld = static_cast<double *>(s.field);
  const double *in = g.take + (static_cast<size_t>(q) * g.nops + r) * 16;
  for (int k = 0; k < s.nv; k++) {
    const double v = in[k];
    if (op.type == GOP_COPY2) {
      double *src = fld + (static_cast<size_t>(op.src_slot) * s.nv + k) * NN + op.src_pos;
      if (v != 0.0) atomicAdd(src, v);
      if (in[8 + k] != 0.0) atomicAdd(src + 1, in[8 + k]);
      continue;
    }
    if (v == 0.0) continue;
    if (op.type == GOP_COPY) {
      atomicAdd(fld + (static_cast<size_t>(op.src_slot) * s.nv + k) * NN + op.src_pos, v);
    } else if (op.type == GOP_SNAP) {
      const GhostSnap sn = g.snaps[op.src_slot];
      atomicAdd(fld + (static_cast<size_t>(sn.slot) * s.nv + k) * NN + sn.pos, v);
    } else {
      double w[4];
      fine_weights(s.kind, k, w);
      for (int p = 0; p < 4; p++) {
        if (w[p] == 0.0) continue;
        size_t at;
        if (op.type == GOP_FINE) {
          const int off = p == 0 ? 0 : (p == 1 ? N : (p == 2 ? 1 : N + 1));
          at = (static_cast<size_t>(op.src_slot) * s.nv + k) * NN + op.src_pos + off;
        } else {  // GOP_SFINE: snapshot rows src_slot .. src_slot + 3
          const GhostSnap sn = g.snaps[op.src_slot + p];
          at = (static_cast<size_t>(sn.slot) * s.nv + k) * NN + sn.pos;
        }
        atomicAdd(fld + at, w[p] * v);
      }
    }
  }
}

// ------------------------------------------------------------- CT2D
struct CtAdjArgs {
  const LeafTask *tasks;
  const InstParams *inst;
  int step;
  // forward values
  const double *Bnew;      // face field after its fill (input of the cell correction)
  const double *qpre;      // cell state before the correction
  // adjoints
  double *aq;              // cell state (in place: post -> pre correction)
  double *aBnew;           // face field written by the face update
  double *aBsrc;           // CT2D's Bi argument
  double *aE;              // EMF
  double *aF, *aG;         // fluxes after their fill
};

// CT2D.cpp:99-120 transposed: q4 += (|b_avg|^2 - q5^2 - q6^2)/2, q5 = bx, q6 = by
template <int NG>
__global__ void k_ct_cell_adj(CtAdjArgs a) {
  constexpr int N = Geo<NG>::N, NN = N * N;
  const LeafTask t = a.tasks[blockIdx.x];
  const double *B = a.Bnew + static_cast<size_t>(t.slot) * 2 * NN;
  const double *qp = a.qpre + static_cast<size_t>(t.slot) * 8 * NN;
  double *aq = a.aq + static_cast<size_t>(t.slot) * 8 * NN;
  double *aB = a.aBnew + static_cast<size_t>(t.slot) * 2 * NN;
  for (int c = threadIdx.x; c < NN; c += blockDim.x) {
    const int i = c % N, j = c / N;
    const int ip = i < N - 1 ? i + 1 : i, ii = ip - 1;
    const int jp = j < N - 1 ? j + 1 : j, jj = jp - 1;
    const double bx = 0.5 * (B[j * N + ip] + B[j * N + ii]);
    const double by = 0.5 * (B[NN + jp * N + i] + B[NN + jj * N + i]);
    const double a4 = aq[4 * NN + c];
    const double lbx = aq[5 * NN + c] + a4 * bx;
    const double lby = aq[6 * NN + c] + a4 * by;
    aq[5 * NN + c] = -a4 * qp[5 * NN + c];
    aq[6 * NN + c] = -a4 * qp[6 * NN + c];
    atomicAdd(aB + j * N + ip, 0.5 * lbx);
    atomicAdd(aB + j * N + ii, 0.5 * lbx);
    atomicAdd(aB + NN + jp * N + i, 0.5 * lby);
    atomicAdd(aB + NN + jj * N + i, 0.5 * lby);
  }
}

// CT2D.cpp:78-92 transposed.  Bx' = s Bsrc (+ s Bold) - s dt/dy (E[i][jp] - E[i][j]),
// By' = ... + s dt/dx (E[ip][j] - E[i][j]), s = 1 (stage 1) or 1/2 (stage 2).
// Adds the EMF adjoint (gathered) and s * aBnew to aBsrc; the caller then
// scales (stage 2) or clears (stage 1) aBnew.
template <int NG>
__global__ void k_ct_face_adj(CtAdjArgs a) {
  constexpr int N = Geo<NG>::N, NN = N * N;
  const LeafTask t = a.tasks[blockIdx.x];
  const double dt = a.inst[t.inst].dt;
  const double s = a.step == 1 ? 1.0 : 0.5;
  const double cx = s * dt * t.rcp_dy, cy = s * dt * t.rcp_dx;
  const double *aBx = a.aBnew + static_cast<size_t>(t.slot) * 2 * NN, *aBy = aBx + NN;
  double *aS = a.aBsrc + static_cast<size_t>(t.slot) * 2 * NN;
  double *aE = a.aE + static_cast<size_t>(t.slot) * NN;
  for (int c = threadIdx.x; c < NN; c += blockDim.x) {
    const int i = c % N, j = c / N;
    double e = 0.0;
    if (j < N - 1) e += cx * aBx[c];
    if (j >= 1 && j - 1 < N - 1) e -= cx * aBx[c - N];
    if (i < N - 1) e -= cy * aBy[c];
    if (i >= 1 && i - 1 < N - 1) e += cy * aBy[c - 1];
    aE[c] += e;
    aS[c] += s * aBx[c];
    aS[NN + c] += s * aBy[c];
  }
}

// CT2D.cpp:16-26 transposed: E[i][j] = (gg5[i-1][j] + gg5[i][j] - ff6[i][j-1]
// - ff6[i][j]) / 4 for i, j >= 1
template <int NG>
__global__ void k_ct_emf_adj(CtAdjArgs a) {
  constexpr int N = Geo<NG>::N, NN = N * N;
  const LeafTask t = a.tasks[blockIdx.x];
  const double *aE = a.aE + static_cast<size_t>(t.slot) * NN;
  double *aF6 = a.aF + static_cast<size_t>(t.slot) * 8 * NN + 6 * NN;
  double *aG5 = a.aG + static_cast<size_t>(t.slot) * 8 * NN + 5 * NN;
  for (int c = threadIdx.x; c < NN; c += blockDim.x) {
    const int i = c % N, j = c / N;
    double g = 0.0, f = 0.0;
    if (i >= 1 && j >= 1) { g += aE[c]; f += aE[c]; }
    if (i + 1 < N && j >= 1) g += aE[c + 1];
    if (j + 1 < N && i >= 1) f += aE[c + N];
    aG5[c] += 0.25 * g;
    aF6[c] -= 0.25 * f;
  }
}

// ------------------------------------------------------------- RK stage
struct StageAdjArgs {
  const LeafTask *tasks;
  const InstParams *inst;
  int step;
  int ntasks;
  const double *W;     // primitive state of the stage (all cells)
  const double *B;     // face field the stage read
  double *aOut;        // adjoint of the stage output (Us or U)
  double *aIn;         // adjoint of the stage input (U or Us)
  const double *aF, *aG;  // flux adjoints after the transposed fill (pre-fill fluxes)
  double *aB;          // adjoint of B (normal face components)
  // per face and variable, the adjoint reaching the primitive state of the
  // stencil cells m-1, m, m+1, m+2 of the face m+1/2: C[dir][q], [slot][8][NN],
  // stored at the face position (cell m+1)
  double *C[2][4];
};

// MC / minmod limiter value and its derivative in r (slopelimiter.cpp:14-27),
// following the branch the forward takes
__device__ __forceinline__ double limiter_d(int lim, double r, double &d) {
  if (lim == LIM_MC) {
    const double a = 2.0 * r, b = 0.5 * (1.0 + r);
    const double c = mmin(a, b), dc = a < b ? 2.0 : 0.5;
    const double e = mmin(c, 2.0), de = c < 2.0 ? dc : 0.0;
    d = 0.0 > e ? 0.0 : de;
    return mmax(0.0, e);
  }
  const double e = mmin(1.0, r), de = 1.0 < r ? 0.0 : 1.0;  // minmod
  d = 0.0 > e ? 0.0 : de;
  return mmax(0.0, e);
}

// celledges.cpp:38-43 for one variable of the face m+1/2 (the states of
// muscl_face, same operations) and their derivatives with respect to
// W[m-1], W[m], W[m+1], W[m+2]: left = l0 W[m-1] + l1 W[m] + l2 W[m+1] to
// first order, right = r0 W[m] + r1 W[m+1] + r2 W[m+2]
struct FaceJac { double left, right, l0, l1, l2, r0, r1, r2; };

__device__ __forceinline__ FaceJac muscl_face_jac(int lim, double wm, double w0, double w1, double w2) {
  const double E = 1.0E-15;
  const double dA = w0 - wm, dB = w1 - w0, dC = w2 - w1;
  FaceJac J;
  double d;
  // left = w0 + phi(dB / (dA + E)) dA / 2
  double phi = limiter_d(lim, limiter_ratio<double>(lim, dB, dA + E), d);
  J.left = w0 + 0.5 * phi * dA;
  double ldA = 0.5 * phi, ldB = 0.0;
  if (d != 0.0) {
    const double inv = 1.0 / (dA + E), q = 0.5 * dA * d * inv;
    ldA -= q * dB * inv;
    ldB = q;
  }
  J.l0 = -ldA;
  J.l1 = 1.0 + ldA - ldB;
  J.l2 = ldB;
  // right = w1 - phi(dB / (dC + E)) dC / 2
  phi = limiter_d(lim, limiter_ratio<double>(lim, dB, dC + E), d);
  J.right = w1 - 0.5 * phi * dC;
  double rdC = -0.5 * phi, rdB = 0.0;
  if (d != 0.0) {
    const double inv = 1.0 / (dC + E), q = 0.5 * dC * d * inv;
    rdC += q * dB * inv;
    rdB = -q;
  }
  J.r0 = -rdB;
  J.r1 = 1.0 + rdB - rdC;
  J.r2 = rdC;
  return J;
}

// One side of a Rusanov face in the x frame (riemannS.cpp:59-108,
// misc.cpp:71-79): the conserved state and the intermediates of the fast
// speed, each evaluated once for the transposed flux.
struct SideAD {
  double q[8];
  double irho, e, pt, A, C, T, D, cf;
};

__device__ __forceinline__ void side_fwd(const double *w, double g, double ig1, SideAD &S) {
  const double rho = w[0], u = w[1], v = w[2], z = w[3], p = w[4], bx = w[5], by = w[6], bz = w[7];
  const double b2 = bx * bx + by * by + bz * bz, t2 = by * by + bz * bz;
  S.irho = 1.0 / rho;
  S.e = p * ig1 + 0.5 * rho * (u * u + v * v + z * z) + 0.5 * b2;
  S.pt = p + 0.5 * b2;
  S.q[0] = rho; S.q[1] = rho * u; S.q[2] = rho * v; S.q[3] = rho * z;
  S.q[4] = S.e; S.q[5] = bx; S.q[6] = by; S.q[7] = bz;
  S.A = g * p * S.irho;
  S.C = b2 * S.irho;
  S.T = t2 * S.irho;
  S.D = sqrt((S.C - S.A) * (S.C - S.A) + 4.0 * S.A * S.T);
  S.cf = sqrt(0.5 * (S.C + S.A + S.D));
}

// adds d/dw of lF.F + lq.q + lcf.cf of one side to lw
__device__ __forceinline__ void side_adj(const double *w, double g, double ig1, const SideAD &S, const double *lF,
                                         const double *lq, double lcf, double *lw) {
  const double rho = w[0], u = w[1], v = w[2], z = w[3], bx = w[5], by = w[6], bz = w[7];
  const double le = lq[4] + lF[4] * u;     // adjoint of e
  const double lpt = lF[1] + lF[4] * u;    // adjoint of pt
  const double v2 = u * u + v * v + z * z;
  double lr = lq[0] + lq[1] * u + lq[2] * v + lq[3] * z + lF[0] * u + lF[1] * u * u + lF[2] * u * v +
              lF[3] * u * z + le * 0.5 * v2;
  double lu = rho * (lq[1] + lF[0]) + 2.0 * rho * u * lF[1] + rho * v * lF[2] + rho * z * lF[3] +
              lF[4] * (S.e + S.pt - bx * bx) + lF[6] * by + lF[7] * bz + le * rho * u;
  double lv = rho * lq[2] + rho * u * lF[2] - lF[4] * bx * by - lF[6] * bx + le * rho * v;
  double lz = rho * lq[3] + rho * u * lF[3] - lF[4] * bx * bz - lF[7] * bx + le * rho * z;
  double lp = le * ig1 + lpt;
  const double lb = le + lpt;
  double lbx = lq[5] + lb * bx - 2.0 * bx * lF[1] - by * lF[2] - bz * lF[3] -
               (2.0 * u * bx + v * by + z * bz) * lF[4] - v * lF[6] - z * lF[7];
  double lby = lq[6] + lb * by - bx * lF[2] - bx * v * lF[4] + u * lF[6];
  double lbz = lq[7] + lb * bz - bx * lF[3] - bx * z * lF[4] + u * lF[7];
  if (lcf != 0.0) {  // cf^2 = (C + A + D) / 2, D^2 = (C - A)^2 + 4 A T
    const double k = lcf / (4.0 * S.cf);
    double lA = k, lC = k, lT = 0.0;
    if (S.D > 0.0) {
      const double kD = k / S.D;
      lA += kD * (2.0 * S.T - (S.C - S.A));
      lC += kD * (S.C - S.A);
      lT = kD * 2.0 * S.A;
    }
    lr -= (S.A * lA + S.C * lC + S.T * lT) * S.irho;
    lp += g * lA * S.irho;
    const double c2 = 2.0 * lC * S.irho, ct = 2.0 * (lC + lT) * S.irho;
    lbx += bx * c2;
    lby += by * ct;
    lbz += bz * ct;
  }
  lw[0] += lr; lw[1] += lu; lw[2] += lv; lw[3] += lz;
  lw[4] += lp; lw[5] += lbx; lw[6] += lby; lw[7] += lbz;
}

// riemannS.cpp:58-116 (Rusanov) transposed for one face in the x frame:
// f = (FL + FR)/2 - max(cfL + |uL|, cfR + |uR|) (qR - qL)/2
__device__ __forceinline__ void rusa_adj(const double *wL, const double *wR, double g, const double *lf,
                                         double *lwL, double *lwR) {
  const double ig1 = 1.0 / (g - 1.0);
  SideAD L, R;
  side_fwd(wL, g, ig1, L);
  side_fwd(wR, g, ig1, R);
  const double a = L.cf + fabs(wL[1]), b = R.cf + fabs(wR[1]);
  const double im = smax(a, b);
  double lF[8], lqL[8], lqR[8], lim = 0.0;
#pragma unroll
  for (int k = 0; k < 8; k++) {
    lF[k] = 0.5 * lf[k];
    lqL[k] = 0.5 * im * lf[k];
    lqR[k] = -0.5 * im * lf[k];
    lim -= 0.5 * lf[k] * (R.q[k] - L.q[k]);
  }
  const double la = a < b ? 0.0 : lim, lb = a < b ? lim : 0.0;
#pragma unroll
  for (int k = 0; k < 8; k++) { lwL[k] = 0.0; lwR[k] = 0.0; }
  lwL[1] += la * sgn(wL[1]);
  lwR[1] += lb * sgn(wR[1]);
  side_adj(wL, g, ig1, L, lF, lqL, la, lwL);
  side_adj(wR, g, ig1, R, lF, lqR, lb, lwR);
}

// MUSCL2D.cpp:24-116 + riemannS + the residual (main.cpp:147-157)
// transposed for one face: the flux adjoint (from CT2D through the fill, plus
// the residual of the face's two cells) becomes the adjoint of the two
// reconstructed states, of the normal face field (added to aB) and, through
// the MUSCL Jacobian, of the primitive state of the four stencil cells (C).
template <int NG>
__global__ void __launch_bounds__(128) k_faces_adj(StageAdjArgs a) {
  using G = Geo<NG>;
  constexpr int N = G::N, NN = G::NN, LO = G::LO, HI = G::HI, NF = G::NF, PER = 2 * NF * NF;
  const size_t e = static_cast<size_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (e >= static_cast<size_t>(a.ntasks) * PER) return;
  const int t = static_cast<int>(e / PER), f = static_cast<int>(e % PER);
  const LeafTask task = a.tasks[t];
  const InstParams ip = a.inst[task.inst];
  const int lim = ip.limiter;
  const size_t base = static_cast<size_t>(task.slot) * 8 * NN;
  const double *W = a.W + base;
  const bool yf = f >= NF * NF;
  const int gi = yf ? f - NF * NF : f;
  const int r = gi / NF, c = gi % NF;
  const int s = yf ? N : 1;
  const int cL = (LO + r) * N + (LO + c);   // cell m of the face m+1/2
  const int kn = yf ? 6 : 5;
  const int fpos = cL + s;
  const double bn = a.B[static_cast<size_t>(task.slot) * 2 * NN + (yf ? NN : 0) + fpos];
  double wl[8], wr[8];
  FaceJac J[8];
#pragma unroll
  for (int k = 0; k < 8; k++) {
    if (k == kn) { wl[k] = wr[k] = bn; continue; }
    const double *w = W + k * NN + cL;
    J[k] = muscl_face_jac(lim, w[-s], w[0], w[s], w[2 * s]);
    wl[k] = J[k].left;
    wr[k] = J[k].right;
  }
  // flux adjoint: CT2D part after the fill, plus the residual of cells m
  // (+1/h) and m+1 (-1/h) when they lie in [LO, HI]
  const double sdt = (a.step == 1 ? 1.0 : 0.5) * ip.dt;
  const double h = yf ? (task.inv_dy != 0.0 ? task.inv_dy : 1.0 / task.dy)
                      : (task.inv_dx != 0.0 ? task.inv_dx : 1.0 / task.dx);
  const int m = LO + (yf ? r : c);          // cell index along the face normal
  const bool hi_in = m + 1 <= HI;
  const double *af = (yf ? a.aG : a.aF) + base + fpos;
  const double *ao = a.aOut + base + cL;
  double lf[8];
#pragma unroll
  for (int k = 0; k < 8; k++) {
    const double r0 = -sdt * ao[k * NN];
    const double r1 = hi_in ? -sdt * ao[k * NN + s] : 0.0;
    lf[k] = af[k * NN] + (r0 - r1) * h;
  }
  double lwl[8], lwr[8];
  if (!yf) {
    rusa_adj(wl, wr, ip.gamma, lf, lwl, lwr);
  } else {  // riemannS.cpp:12-23 / 47-55: swap (u, v) and (Bx, By)
    double l2[8], r2[8], f2[8], a2[8], b2[8];
#pragma unroll
    for (int k = 0; k < 8; k++) { l2[k] = wl[k]; r2[k] = wr[k]; f2[k] = lf[k]; }
    l2[1] = wl[2]; l2[2] = wl[1]; r2[1] = wr[2]; r2[2] = wr[1];
    l2[5] = wl[6]; l2[6] = wl[5]; r2[5] = wr[6]; r2[6] = wr[5];
    f2[1] = lf[2]; f2[2] = lf[1]; f2[5] = lf[6]; f2[6] = lf[5];
    rusa_adj(l2, r2, ip.gamma, f2, a2, b2);
#pragma unroll
    for (int k = 0; k < 8; k++) { lwl[k] = a2[k]; lwr[k] = b2[k]; }
    lwl[1] = a2[2]; lwl[2] = a2[1]; lwr[1] = b2[2]; lwr[2] = b2[1];
    lwl[5] = a2[6]; lwl[6] = a2[5]; lwr[5] = b2[6]; lwr[6] = b2[5];
  }
  // the normal component of both states is the face field (MUSCL2D.cpp:48-51)
  a.aB[static_cast<size_t>(task.slot) * 2 * NN + (yf ? NN : 0) + fpos] += lwl[kn] + lwr[kn];
  const int d = yf ? 1 : 0;
  double *c0 = a.C[d][0] + base + fpos, *c1 = a.C[d][1] + base + fpos;
  double *c2 = a.C[d][2] + base + fpos, *c3 = a.C[d][3] + base + fpos;
#pragma unroll
  for (int k = 0; k < 8; k++) {
    if (k == kn) continue;
    const double L = lwl[k], R = lwr[k];
    c0[k * NN] = J[k].l0 * L;                  // cell m-1
    c1[k * NN] = J[k].l1 * L + J[k].r0 * R;    // cell m
    c2[k * NN] = J[k].l2 * L + J[k].r1 * R;    // cell m+1
    c3[k * NN] = J[k].r2 * R;                  // cell m+2
  }
}

// Per cell: the primitive-state adjoint gathered from the (up to 8) faces
// whose reconstruction read the cell, the transpose of U2W
// (meshblock.cpp:119-145) added to aIn, and the RK combine
// (main.cpp:147-157 / 179-189) transposed (aIn += s aOut; aOut -> the old
// state's adjoint).  Face m+1/2 (m in [LO, HI]) gives cell m-1+q its C[q].
template <int NG>
__global__ void __launch_bounds__(256) k_cells_adj(StageAdjArgs a) {
  using G = Geo<NG>;
  constexpr int N = G::N, NN = G::NN, LO = G::LO, HI = G::HI;
  const size_t e = static_cast<size_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (e >= static_cast<size_t>(a.ntasks) * NN) return;
  const int t = static_cast<int>(e / NN), c = static_cast<int>(e % NN);
  const int i = c % N, j = c / N;
  const LeafTask task = a.tasks[t];
  const double gamma = a.inst[task.inst].gamma;
  const size_t base = static_cast<size_t>(task.slot) * 8 * NN;
  const bool xrow = j >= LO && j <= HI, ycol = i >= LO && i <= HI;
  // faces m = pos + 1 - q: valid when LO <= m <= HI
  bool vx[4], vy[4];
#pragma unroll
  for (int q = 0; q < 4; q++) {
    vx[q] = xrow && i + 1 - q >= LO && i + 1 - q <= HI;
    vy[q] = ycol && j + 1 - q >= LO && j + 1 - q <= HI;
  }
  double lw[8];
#pragma unroll
  for (int k = 0; k < 8; k++) {
    double acc = 0.0;
#pragma unroll
    for (int q = 0; q < 4; q++) {
      if (k != 5 && vx[q]) acc += a.C[0][q][base + k * NN + c + 2 - q];
      if (k != 6 && vy[q]) acc += a.C[1][q][base + k * NN + c + (2 - q) * N];
    }
    lw[k] = acc;
  }
  const double *W = a.W + base;
  const double rho = W[c], u = W[NN + c], v = W[2 * NN + c], z = W[3 * NN + c];
  const double gm = gamma - 1.0;
  double g[8];
  g[0] = lw[0] - (lw[1] * u + lw[2] * v + lw[3] * z) / rho + lw[4] * gm * 0.5 * (u * u + v * v + z * z);
  g[1] = lw[1] / rho - lw[4] * gm * u;
  g[2] = lw[2] / rho - lw[4] * gm * v;
  g[3] = lw[3] / rho - lw[4] * gm * z;
  g[4] = lw[4] * gm;
#pragma unroll
  for (int k = 5; k < 8; k++) g[k] = lw[k] - lw[4] * gm * W[k * NN + c];
  const double sk = a.step == 1 ? 1.0 : 0.5;
#pragma unroll
  for (int k = 0; k < 8; k++) {
    const size_t idx = base + k * NN + c;
    const double o = a.aOut[idx];
    a.aIn[idx] += sk * o + g[k];
    a.aOut[idx] = a.step == 1 ? 0.0 : 0.5 * o;
  }
}

}  // namespace amr
