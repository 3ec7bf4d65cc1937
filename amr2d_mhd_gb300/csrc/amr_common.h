// Shared definitions of the host engine and the sm_103a kernels.
#pragma once

#include <stdint.h>

namespace amr {

constexpr int NI = 16;     // interior cells per block edge (input.txt "16 16 8")
constexpr int NVAR = 8;    // rho, rho u, rho v, rho w, E, Bx, By, Bz (meshblock.cpp:19-21)
constexpr double EPS = 1.0E-15;  // defs.hpp:16 (DOUBLE_PREC)

// limiter ids (slopelimiter.cpp:8-48) and reconstruction families (MUSCL2D.cpp:24-34)
enum Limiter { LIM_1ST = 0, LIM_NOSL, LIM_MINMOD, LIM_VANLEER, LIM_SUPERBEE, LIM_MC, LIM_KOREN,
               LIM_CADA3RD, LIM_WENO3, LIM_WENO5 };
enum Recon { REC_MUSCL = 0, REC_WENO3 = 1, REC_WENO5 = 2 };
// Riemann solvers (riemannS.cpp:30-44)
enum Flux { FLX_RUSA = 0, FLX_HLLE, FLX_HLLC, FLX_HLLD, FLX_ROE };

// device error word: first failure wins (code, block, i, j)
enum DevErr { DERR_NONE = 0, DERR_PRESSURE = 1, DERR_NAN = 2, DERR_HLLC = 3, DERR_REFINE_NAN = 4, DERR_TIMEOUT = 5,
              DERR_PSI = 6 };
struct DevError {
  int code;
  int blk;
  int i, j;
  double value;
};

// One leaf block to process: its physical slot and the instance it belongs to.
struct LeafTask {
  int slot;
  int inst;
  double dx, dy;
  // 1/dx and 1/dy when dx, dy are powers of two (then x/dx == x*(1/dx)
  // exactly, and the residual multiplies instead of dividing); 0 otherwise
  double inv_dx, inv_dy;
  // 1./dx and 1./dy rounded as the device division rounds them (IEEE), for
  // the formulas that multiply by the rounded reciprocal (CT2D.cpp:80,86)
  double rcp_dx, rcp_dy;
  int flags;      // TASK_DIFFUSE
  // the block's share of the step's compiled ghost fill, for fills fused into
  // the step's kernels: the ops that write its ghost cells, and the
  // snapshots of its cells (ranges of the device program)
  int op_count;
  int op_begin;
  int snap_begin;
  int snap_count;
  int pad;
};
// the block takes diffusivity.cpp after stage 2 (main.cpp:190-193)
constexpr int TASK_DIFFUSE = 1;

// 1/v if v is a power of two (exact reciprocal), else 0
inline double exact_reciprocal(double v) {
  int e = 0;
  const double m = __builtin_frexp(v, &e);
  return (m == 0.5) ? 1.0 / v : 0.0;
}

// Per-instance scalars read by the kernels (kept in device memory so that a
// captured CUDA graph sees the values of the current step).
struct InstParams {
  double gamma;
  double dt;      // dom.dt of the current step
  int limiter;
  int ct_type;    // 2 = upwind-switched EMF (CT2D.cpp:28-75), else the average
};

// One gather of a compiled ghost fill (see ghost_compile.cpp).  The same op
// list serves the cell, face and edge fills: only the fine-to-coarse value
// depends on the kind of field, and the kernel applies it per kind.
//   COPY:   dst <- src                      (value before the fill)
//   SNAP:   dst <- snapshot row src_slot    (a pre-fill value of a cell the
//                                            same fill overwrites; saved first)
//   FINE:   dst <- fine-to-coarse value of the 2x2 patch with lower-left src:
//             cell  0.25*(s(i,j)+s(i,j+1)+s(i+1,j)+s(i+1,j+1))   boundary.cpp:48
//             face  0.5*(s(i,j)+s(i,j+1)) for k==0,
//                   0.5*(s(i,j)+s(i+1,j)) for k>0                boundaryfc.cpp:48
//             edge  s(i,j)                                       boundaryec.cpp:46
//   SFINE:  the same from four saved pre-fill values (snapshot rows src_slot..
//           src_slot+3 in the order (i,j) (i,j+1) (i+1,j) (i+1,j+1))
// GOP_COPY2: two horizontally adjacent cells (dst_pos, dst_pos + 1) from
// (src_pos, src_pos + 1) of one source block; both positions even, so the
// pair is one aligned 8-byte (float) or 16-byte (double) access.
enum GhostOpType : uint8_t { GOP_COPY = 0, GOP_SNAP = 1, GOP_FINE = 2, GOP_SFINE = 3, GOP_NOP = 4, GOP_COPY2 = 5 };
struct GhostOp {
  int dst_slot;
  int src_slot;     // physical slot, or first snapshot row for SNAP / SFINE
  int16_t dst_pos;  // j * N + i within the block plane
  int16_t src_pos;
  uint8_t type;     // GhostOpType
  uint8_t pad[3];
};
// A pre-fill cell saved before a fill runs (all variables of the field).
struct GhostSnap {
  int slot;
  int pos;
};

// refine (dad -> 4 sons) or coarsen (4 sons -> dad) in physical slots
struct TreeOp {
  int dad;
  int son[4];
  int inst;
};

}  // namespace amr
