// Fused RK stage of one leaf block: MUSCL2D.cpp:13-121 (cons2prim,
// reconstruction, CT normal-B override, Riemann fluxes) followed by the
// residual and RK2ndv1 update of main.cpp:147-157 / 179-189.
//
// One CTA per leaf block.  Shared memory holds the primitive state of the
// whole block (with ghosts) and the x / y face fluxes that the residual
// needs; the fluxes also go to global memory (ff, gg), which the ghost fill
// and the CT EMF read next.
#pragma once

#include "amr_common.h"
#include "ghost.cuh"
#include "physics.cuh"

namespace amr {

template <int NG>
struct Geo {
  static constexpr int N = NI + 2 * NG;   // block edge with ghosts (nx of the reference)
  static constexpr int NN = N * N;
  static constexpr int LO = NG - 1;       // nxminb
  static constexpr int HI = NG + NI - 1;  // nxmax
  static constexpr int NF = NI + 1;       // faces per row computed by MUSCL2D (17)
  static constexpr int NFX = NI + 2;      // plus the stale face at LO (18)
};

struct StageArgs {
  const LeafTask *tasks;
  const InstParams *inst;
  const void *qin;    // U (stage 1) or Us (stage 2)
  void *qout;         // Us (stage 1) or U (stage 2, read-modify-write)
  const double *B;    // Bi (stage 1) or Bis (stage 2)
  void *ff;
  void *gg;
  DevError *err;
  unsigned *ctr;      // [2] block counter and finished-CTA counter of k_stage_dyn (zero between launches)
  int step;
  int ntasks;         // leaf blocks (k_stage_dyn)
  FillFuse fuse;      // fused fills: the qin fill gathered first (mirrored in
                      // shared memory), the flux fill's snapshots saved last
};

// First statement of every kernel of the step: when the kernel was launched
// as a programmatic dependent of the previous one (Method::pdl), wait until
// that grid has completed and its memory is visible; without that launch
// attribute it returns at once.  The kernel may then be scheduled while its
// predecessor drains, which hides most of the gap between the step's many
// small kernels.
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }

__device__ __forceinline__ void dev_fail(DevError *e, int code, int blk, int i, int j, double v) {
  if (atomicCAS(&e->code, 0, code) == 0) {
    e->blk = blk;
    e->i = i;
    e->j = j;
    e->value = v;
  }
}

// floor of the pressure recovered by the FP32 path (code units)
constexpr double kPressureFloor = 1.0e-10;

// meshblock.cpp:119-179 for one cell; the FP32 path recovers the pressure in
// FP64 from the FP32 conserved state and floors it (positivity fix).
template <typename S>
__device__ __forceinline__ void cons2prim_cell(const S *u, S *w, double gamma);

template <>
__device__ __forceinline__ void cons2prim_cell<double>(const double *u, double *w, double g) {
  w[0] = u[0];
  w[1] = u[1] / u[0];
  w[2] = u[2] / u[0];
  w[3] = u[3] / u[0];
  double p = (g - 1) * (u[4] - 0.5 * w[0] * (w[1] * w[1] + w[2] * w[2] + w[3] * w[3]));
  w[5] = u[5];
  w[6] = u[6];
  w[7] = u[7];
  w[4] = p - (g - 1) * (0.5 * (u[5] * u[5] + u[6] * u[6] + u[7] * u[7]));
}

// a^2 + b^2 + c^2 of FP32 values as an unevaluated sum hi + lo, exact to
// about 2^-48 relative: each square split exactly by an FMA (Dekker's
// product) and the partial sums by Knuth's TwoSum, with the error terms
// summed in FP32.  The _rn intrinsics keep the compiler from fusing or
// reordering the steps.
__device__ __forceinline__ void sum_sq3(float a, float b, float c, float &hi, float &lo) {
  const float pa = __fmul_rn(a, a), pb = __fmul_rn(b, b), pc = __fmul_rn(c, c);
  const float ea = __fmaf_rn(a, a, -pa), eb = __fmaf_rn(b, b, -pb), ec = __fmaf_rn(c, c, -pc);
  const float s1 = __fadd_rn(pa, pb), v1 = __fsub_rn(s1, pa);
  const float t1 = __fadd_rn(__fsub_rn(pa, __fsub_rn(s1, v1)), __fsub_rn(pb, v1));
  const float s2 = __fadd_rn(s1, pc), v2 = __fsub_rn(s2, s1);
  const float t2 = __fadd_rn(__fsub_rn(s1, __fsub_rn(s2, v2)), __fsub_rn(pc, v2));
  hi = s2;
  lo = __fadd_rn(__fadd_rn(__fadd_rn(ea, eb), ec), __fadd_rn(t1, t2));
}

// FP32 path: the pressure recovered from the total energy in FP64 (the
// cancellation E - |m|^2/2rho - |B|^2/2 is where FP32 loses digits).  The
// sums of squares |m|^2 and |B|^2 and the quotient |m|^2/rho come from the
// FP32 pipe as hi + lo pairs (sum_sq3, and the product with 1/rho = ir + rl),
// accurate to ~2^-45, and are widened to FP64 only for E - (|m|^2/rho +
// |B|^2)/2 and the factor gamma - 1.  On this GPU FP64 runs at 1/64 of the
// FP32 rate: this takes a third of the FP64 operations of squaring, summing
// and dividing in FP64.  AMR_PRESSURE_DF=1: |m|^2/rho with 1/rho refined by
// one FP64 Newton step instead.
// The velocities are the FP32 momenta times the FP32 reciprocal.  (A
// component above ~1.8e19 overflows its FP32 square; such a state is out of
// the FP32 path's range in any case.)  AMR_PRESSURE_DF=0 restores the FP64
// squares and sums.
#ifndef AMR_PRESSURE_DF
#define AMR_PRESSURE_DF 2
#endif
template <>
__device__ __forceinline__ void cons2prim_cell<float>(const float *u, float *w, double g) {
  const float ir = 1.0f / u[0];
#if AMR_PRESSURE_DF == 2
  // |m|^2 / rho as hi + lo on the FP32 pipe too: 1/rho = ir + rl (rl from the
  // FMA residual 1 - rho*ir, ~2^-45 relative), the product of the two pairs
  // with Dekker's exact error term
  const float rl = __fmul_rn(__fmaf_rn(-u[0], ir, 1.0f), ir);
  float mh, ml, bh, bl;
  sum_sq3(u[1], u[2], u[3], mh, ml);
  sum_sq3(u[5], u[6], u[7], bh, bl);
  const float kh = __fmul_rn(mh, ir);
  const float kl = __fadd_rn(__fmaf_rn(mh, ir, -kh), __fadd_rn(__fmul_rn(mh, rl), __fmul_rn(ml, ir)));
  double p = (g - 1) * (static_cast<double>(u[4]) -
                        0.5 * ((static_cast<double>(kh) + static_cast<double>(kl)) +
                               (static_cast<double>(bh) + static_cast<double>(bl))));
#elif AMR_PRESSURE_DF
  double ird = static_cast<double>(ir);
  ird = __fma_rn(ird, __fma_rn(-static_cast<double>(u[0]), ird, 1.0), ird);
  float mh, ml, bh, bl;
  sum_sq3(u[1], u[2], u[3], mh, ml);
  sum_sq3(u[5], u[6], u[7], bh, bl);
  const double m2 = static_cast<double>(mh) + static_cast<double>(ml);
  const double b2 = static_cast<double>(bh) + static_cast<double>(bl);
  double p = (g - 1) * (static_cast<double>(u[4]) - 0.5 * (m2 * ird + b2));
#else
  double ird = static_cast<double>(ir);
  ird = ird * (2.0 - static_cast<double>(u[0]) * ird);
  const double mx = u[1], my = u[2], mz = u[3];
  const double bx = u[5], by = u[6], bz = u[7];
  double p = (g - 1) * (static_cast<double>(u[4]) - 0.5 * (mx * mx + my * my + mz * mz) * ird) -
             (g - 1) * (0.5 * (bx * bx + by * by + bz * bz));
#endif
  // positivity fix of the FP32 path: the FP32 conserved state can put the
  // recovered pressure below zero where the FP64 path stays positive
  if (!(p > kPressureFloor)) p = kPressureFloor;
  w[0] = u[0];
  w[1] = u[1] * ir;
  w[2] = u[2] * ir;
  w[3] = u[3] * ir;
  w[4] = static_cast<float>(p);
  w[5] = u[5];
  w[6] = u[6];
  w[7] = u[7];
}

// FP32 fused stage: 320 threads per CTA (the 2 x 17 x 17 = 578 faces of a
// block in two rounds; 256 threads take three, the last a quarter full),
// compiled for 3 resident CTAs per SM (64 registers, ~120 B of spills to L1).
// Timed on the 64-rotor FP32 batch (one GB300, 20 steps): 5.17 ms per step
// against 5.52 ms at 256 threads / 4 CTAs, 5.57 ms at 320 / 2 CTAs (96
// registers, no spills); the 512-blast batch 24.7 against 25.1 and 27.8 ms.
#ifndef AMR_STAGE_F32_MINB
#define AMR_STAGE_F32_MINB 3
#endif
#ifndef AMR_STAGE_F32_THREADS
#define AMR_STAGE_F32_THREADS 320
#endif
// 1: the FP32 fused stage keeps the block's conserved state in shared memory
// beside the primitive state, so the RK update does not read it again (no
// gain measured: 5.60 against 5.52 ms per step of the 64-rotor batch)
#ifndef AMR_STAGE_F32_KEEPU
#define AMR_STAGE_F32_KEEPU 0
#endif

// ------------------------------------------------------------ bulk staging
// One thread issues a bulk copy (TMA, cp.async.bulk) of `bytes` contiguous
// bytes from global to shared memory, completing on an mbarrier; every
// thread then waits for the phase with a bounded spin.  Both addresses and
// the size are multiples of 16 bytes (checked by the caller's layout).
constexpr long kBulkSpinLimit = 1L << 26;

__device__ __forceinline__ uint32_t smem_u32(const void *p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void bulk_stage_issue(void *dst, const void *src, uint32_t bytes, uint64_t *bar) {
  const uint32_t b = smem_u32(bar);
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(b), "r"(bytes) : "memory");
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
               ::"r"(smem_u32(dst)), "l"(src), "r"(bytes), "r"(b)
               : "memory");
}

// true once the phase completed; false after the spin limit
__device__ __forceinline__ bool bulk_stage_wait(uint64_t *bar, uint32_t phase) {
  const uint32_t b = smem_u32(bar);
  for (long it = 0; it < kBulkSpinLimit; it++) {
    uint32_t done;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(done)
        : "r"(b), "r"(phase)
        : "memory");
    if (done) return true;
  }
  return false;
}

// resident CTAs per SM the fused stage kernel is compiled for: the FP32
// instantiation trades registers for occupancy (it is latency-bound)
template <typename S> struct StageMinBlocks { static constexpr int value = 1; };
template <> struct StageMinBlocks<float> { static constexpr int value = AMR_STAGE_F32_MINB; };
template <typename S> struct StageThreads { static constexpr int value = 256; };
template <> struct StageThreads<float> { static constexpr int value = AMR_STAGE_F32_THREADS; };
template <typename S> struct StageKeepU { static constexpr bool value = false; };
template <> struct StageKeepU<float> { static constexpr bool value = AMR_STAGE_F32_KEEPU != 0; };

// One leaf block of the fused stage: task `ti`, its conserved state staged
// into shared memory by a bulk copy completing on `bar` (initialised by the
// caller) in phase `phase`.  Returns false (after recording DERR_TIMEOUT and
// letting the copy land) when the bounded wait gave up; the decision is the
// same in every thread of the CTA.
template <int NG, int RECON, int FLUX, typename S>
__device__ __forceinline__ bool stage_block(const StageArgs &a, int ti, uint64_t *bar, uint32_t phase) {
  using G = Geo<NG>;
  using T = S;
  constexpr int N = G::N, NN = G::NN, LO = G::LO, HI = G::HI, NF = G::NF, NFX = G::NFX;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T *sW = reinterpret_cast<T *>(smem_raw);   // [8][NN]
  T *sFx = sW + 8 * NN;                      // [8][NF][NFX]   face i = LO + col, row j = LO + r
  T *sFy = sFx + 8 * NF * NFX;               // [8][NFX][NF]   face j = LO + row, col i = LO + c
  constexpr bool KEEPU = StageKeepU<S>::value;
  S *sU = KEEPU ? sFy + 8 * NFX * NF : sW;   // [8][NN] the conserved state (KEEPU), else staged in sW

  const LeafTask task = a.tasks[ti];
  const InstParams ip = a.inst[task.inst];
  const size_t base = static_cast<size_t>(task.slot) * 8 * NN;
  const S *Q = static_cast<const S *>(a.qin) + base;
  S *ff = static_cast<S *>(a.ff) + base;
  S *gg = static_cast<S *>(a.gg) + base;
  const double *Bx = a.B + static_cast<size_t>(task.slot) * 2 * NN;
  const double *By = Bx + NN;
  const int tid = threadIdx.x, nthr = blockDim.x;

  // 0. the block's conserved state (8 planes, contiguous) into shared memory by TMA
  static_assert((8 * NN * sizeof(S)) % 16 == 0, "bulk copies move multiples of 16 bytes");
  if (tid == 0) bulk_stage_issue(sU, Q, static_cast<uint32_t>(8 * NN * sizeof(S)), bar);
  // fused fill: each thread's first gather is loaded while the copy is in flight
  const FillPre pre = fill_prefetch<N>(a.fuse, task, tid);
  const bool late = !bulk_stage_wait(bar, phase);
  if (__syncthreads_or(late)) {
    if (tid == 0) dev_fail(a.err, DERR_TIMEOUT, task.slot, 0, 0, 0.0);
    bulk_stage_wait(bar, phase);  // let the copy land before the CTA's shared memory is released
    return false;
  }
  // fused fill: the block's ghost cells of qin (and of B), into global memory
  // and over the staged copy, which held the values from before the fill
  if (a.fuse.apply.nseg) {
    fill_apply_task_after<N, S>(a.fuse, task, tid, nthr, sU, pre);
    __syncthreads();
  }

  // 1. primitive variables of every cell (U2W / Us2W), with the traps (in
  // place unless the conserved state is kept)
  for (int c = tid; c < NN; c += nthr) {
    S u[8], w[8];
#pragma unroll
    for (int k = 0; k < 8; k++) u[k] = sU[k * NN + c];
    cons2prim_cell<S>(u, w, ip.gamma);
#pragma unroll
    for (int k = 0; k < 8; k++) sW[k * NN + c] = w[k];
    const int i = c % N, j = c / N;
    if (w[4] <= T(0) && i > LO && i < HI + 1 && j > LO && j < HI + 1)
      dev_fail(a.err, DERR_PRESSURE, task.slot, i, j, static_cast<double>(w[4]));
    bool bad = false;
#pragma unroll
    for (int k = 0; k < 8; k++) bad |= bits_nan(w[k]);
    if (bad) dev_fail(a.err, DERR_NAN, task.slot, i, j, 0.0);
  }
  // fluxes MUSCL2D does not recompute: the x face at LO and the y face at LO
  // (their values come from the previous ghost fill of ff / gg)
  for (int e = tid; e < 8 * NF; e += nthr) {
    const int k = e / NF, r = e % NF;
    sFx[(k * NF + r) * NFX + 0] = ff[k * NN + (LO + r) * N + LO];
    sFy[(k * NFX + 0) * NF + r] = gg[k * NN + LO * N + (LO + r)];
  }
  __syncthreads();

  // 2. Riemann fluxes at x faces (i+1/2, j), i in [LO, HI], and y faces
  const T gamma = static_cast<T>(ip.gamma);
  const int lim = ip.limiter;
  for (int f = tid; f < 2 * NF * NF; f += nthr) {
    const bool yf = f >= NF * NF;
    const int g = yf ? f - NF * NF : f;
    const int r = g / NF, c = g % NF;
    // cell-index stride along the face normal and the left cell of the face
    int s, cL;
    if (!yf) { s = 1; cL = (LO + r) * N + (LO + c); }        // face between (LO+c) and (LO+c+1), row LO+r
    else { s = N; cL = (LO + r) * N + (LO + c); }             // face between rows LO+r and LO+r+1, column LO+c
    const int kn = yf ? 6 : 5;                                // normal B component
    T wl[8], wr[8];
#pragma unroll
    for (int k = 0; k < 8; k++) {
      if (k == kn) continue;
      const T *w = sW + k * NN + cL;
      if (RECON == REC_MUSCL) {
        const T wm = w[-s], w0 = w[0], w1 = w[s], w2 = w[2 * s];
        muscl_face<T>(lim, w0, w1, w0 - wm, w1 - w0, w2 - w1, static_cast<T>(yf ? task.dy : task.dx),
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
    // CT: the normal component is the face value (MUSCL2D.cpp:48-51)
    const int fpos = cL + s;  // face index of the reference = the right cell
    const T bn = static_cast<T>(yf ? By[fpos] : Bx[fpos]);
    wl[kn] = bn;
    wr[kn] = bn;
    T fl[8];
    int rc;
    if (!yf) {
      rc = riemann<FLUX, T>(wl, wr, gamma, fl);
    } else {  // riemannS.cpp:12-23, 47-55: rotate y into x and back
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
    bool bad = false;
#pragma unroll
    for (int k = 0; k < 8; k++) {
      bad |= bits_nan(fl[k]);
      if (!yf) {
        sFx[(k * NF + r) * NFX + (c + 1)] = fl[k];
        ff[k * NN + fpos] = fl[k];
      } else {
        sFy[(k * NFX + (r + 1)) * NF + c] = fl[k];
        gg[k * NN + fpos] = fl[k];
      }
    }
    if (bad) dev_fail(a.err, DERR_NAN, task.slot, fpos % N, fpos / N, 0.0);
  }
  __syncthreads();

  // 3. residual on [LO, HI]^2 (zero elsewhere) and the RK stage on every cell
  const T dx = static_cast<T>(task.dx), dy = static_cast<T>(task.dy), dt = static_cast<T>(ip.dt);
  S *out = static_cast<S *>(a.qout) + base;
  for (int e = tid; e < 8 * NN; e += nthr) {
    const int k = e / NN, c = e % NN;
    const int i = c % N, j = c / N;
    T res = T(0.);
    if (i >= LO && i <= HI && j >= LO && j <= HI) {
      const int cx = i - LO, r = j - LO;
      res = (sFx[(k * NF + r) * NFX + cx + 1] - sFx[(k * NF + r) * NFX + cx]) / dx +
            (sFy[(k * NFX + r + 1) * NF + cx] - sFy[(k * NFX + r) * NF + cx]) / dy;
    }
    const T q = KEEPU ? sU[e] : Q[e];
    if (a.step == 1) out[e] = q - dt * res;                         // Us = U - dt res
    else out[e] = T(0.5) * (out[e] + q - dt * res);                 // U = (U + Us - dt res)/2
  }
  // fused fill: snapshots of the next fill (ff, gg and B, whose writes by
  // this CTA precede the barrier after step 2)
  if (a.fuse.save.nseg) fill_save_task<N>(a.fuse, task, tid, nthr);
  return true;
}

__device__ __forceinline__ void stage_bar_init(uint64_t *bar) {
  if (threadIdx.x == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(1) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();
}

// one CTA per leaf block
template <int NG, int RECON, int FLUX, typename S>
__global__ void __launch_bounds__(StageThreads<S>::value, StageMinBlocks<S>::value) k_stage(StageArgs a) {
  pdl_wait();
  __shared__ __align__(8) uint64_t bar;
  stage_bar_init(&bar);
  stage_block<NG, RECON, FLUX, S>(a, blockIdx.x, &bar, 0);
}

// persistent: a grid of the CTAs the SMs hold at once sweeps the leaf list of
// all instances and levels, each CTA claiming the next block from a global
// counter (the mbarrier phase alternates per block); the last CTA to finish
// zeroes the counters for the next launch
template <int NG, int RECON, int FLUX, typename S>
__global__ void __launch_bounds__(StageThreads<S>::value, StageMinBlocks<S>::value) k_stage_dyn(StageArgs a) {
  pdl_wait();
  __shared__ __align__(8) uint64_t bar;
  __shared__ int next;
  stage_bar_init(&bar);
  for (uint32_t it = 0;; it++) {
    if (threadIdx.x == 0) next = static_cast<int>(atomicAdd(&a.ctr[0], 1u));
    __syncthreads();
    const int ti = next;
    if (ti >= a.ntasks) break;
    if (!stage_block<NG, RECON, FLUX, S>(a, ti, &bar, it & 1u)) break;
    __syncthreads();  // shared memory free for the next block's copy
  }
  if (threadIdx.x == 0) {
    __threadfence();
    if (atomicAdd(&a.ctr[1], 1u) == gridDim.x - 1) {
      a.ctr[0] = 0;
      a.ctr[1] = 0;
    }
  }
}

template <int NG, typename S>
constexpr int stage_smem_bytes() {
  using G = Geo<NG>;
  return static_cast<int>(sizeof(S)) * ((StageKeepU<S>::value ? 16 : 8) * G::NN + 2 * 8 * G::NF * G::NFX);
}

}  // namespace amr
