// Device side of the compiled ghost fills (ghost_compile.cpp): the gather of
// one op, the stand-alone fill launch, and the fused form in which a fill's
// gathers run in the kernel that consumes the filled field and its
// snapshots in the kernel before it.
#pragma once

#include <stddef.h>

#include <type_traits>

#include "amr_common.h"

namespace amr {

// One compiled program (ops + snapshots) serves every field; a launch applies
// it to up to kMaxSeg fields at once.
constexpr int kMaxSeg = 3;
struct GhostSeg {
  void *field;
  int nv;
  int kind;           // FILL_CC / FILL_FC / FILL_EC (ghost_compile.hpp)
  int f32;            // field stored as float
};
struct GhostLaunch {
  const GhostOp *ops;
  const GhostSnap *snaps;
  int nops, nsnaps;
  GhostSeg seg[kMaxSeg];
  int nseg;
  double *snapbuf;    // [nseg][nsnaps][8]
  // variable rows of the launch: segment q owns rows [row0[q], row0[q+1]);
  // set by launch_ghost
  int row0[kMaxSeg + 1];
};

// A fill kernel runs on a 2-D grid: blockIdx.y is the variable row, so that
// consecutive threads take consecutive items (ops or snapshots) of the same
// variable and every load of an item is independent of the others.  The
// segment is picked with constant indices into the parameter block.
__device__ __forceinline__ GhostSeg ghost_seg(const GhostLaunch &g, int row, int &q, int &k) {
  GhostSeg s = g.seg[0];
  q = 0;
  k = row;
  if (g.nseg > 1 && row >= g.row0[1]) { s = g.seg[1]; q = 1; k = row - g.row0[1]; }
  if (g.nseg > 2 && row >= g.row0[2]) { s = g.seg[2]; q = 2; k = row - g.row0[2]; }
  return s;
}

// fine-to-coarse value of one variable from the patch (i,j) (i,j+1) (i+1,j)
// (i+1,j+1): boundary.cpp:48 / boundaryfc.cpp:48 / boundaryec.cpp:46
template <typename F>
__device__ __forceinline__ F fine_value(int kind, int k, F a00, F a01, F a10, F a11) {
  F v = F(0.);
  if (kind == 0) {
    v += a00; v += a01; v += a10; v += a11;
    return F(0.25) * v;
  }
  if (kind == 1) {
    v += a00;
    v += k == 0 ? a01 : a10;
    return F(0.5) * v;
  }
  return a00;
}

// the value(s) of variable k of one gather, computed in the field's type F
// (a pair gives two); and their store to the destination and, when `tile` is
// not null, to the destination block's copy of the field in shared memory
// ([nv][N*N])
template <int N, typename F>
__device__ __forceinline__ void ghost_gather(const GhostSeg &s, const GhostOp &op, int k, const double *snap, F &v0,
                                             F &v1) {
  constexpr int NN = N * N;
  const F *fld = static_cast<const F *>(s.field);
  if (op.type == GOP_COPY2) {  // even positions in an even-sized plane: aligned pair
    using P2 = typename std::conditional<sizeof(F) == 4, float2, double2>::type;
    const P2 v =
        *reinterpret_cast<const P2 *>(fld + (static_cast<size_t>(op.src_slot) * s.nv + k) * NN + op.src_pos);
    v0 = v.x;
    v1 = v.y;
    return;
  }
  if (op.type == GOP_COPY || op.type == GOP_FINE) {
    const F *c = fld + (static_cast<size_t>(op.src_slot) * s.nv + k) * NN + op.src_pos;
    v0 = op.type == GOP_COPY ? c[0] : fine_value<F>(s.kind, k, c[0], c[N], c[1], c[1 + N]);
  } else {
    const double *r = snap + static_cast<size_t>(op.src_slot) * 8 + k;
    v0 = op.type == GOP_SNAP ? static_cast<F>(r[0])
                             : fine_value<F>(s.kind, k, static_cast<F>(r[0]), static_cast<F>(r[8]),
                                             static_cast<F>(r[16]), static_cast<F>(r[24]));
  }
}

template <int N, typename F>
__device__ __forceinline__ void ghost_put(const GhostSeg &s, const GhostOp &op, int k, F v0, F v1, F *tile) {
  constexpr int NN = N * N;
  F *dst = static_cast<F *>(s.field) + (static_cast<size_t>(op.dst_slot) * s.nv + k) * NN + op.dst_pos;
  if (op.type == GOP_COPY2) {
    using P2 = typename std::conditional<sizeof(F) == 4, float2, double2>::type;
    P2 v;
    v.x = v0;
    v.y = v1;
    *reinterpret_cast<P2 *>(dst) = v;
    if (tile) *reinterpret_cast<P2 *>(tile + k * NN + op.dst_pos) = v;
    return;
  }
  *dst = v0;
  if (tile) tile[k * NN + op.dst_pos] = v0;
}

// variable k of one gather (`tile` as for ghost_put)
template <int N, typename F>
__device__ __forceinline__ void ghost_apply_one(const GhostSeg &s, const GhostOp &op, int k, const double *snap,
                                                F *tile = nullptr) {
  F v0, v1 = F(0.);
  ghost_gather<N, F>(s, op, k, snap, v0, v1);
  ghost_put<N, F>(s, op, k, v0, v1, tile);
}

// ------------------------------------------------------------ fused fills
// The compiled program is grouped by block: the ops that write block b's
// ghost cells are ops[op_begin, op_begin + op_count) of b's LeafTask, and
// the snapshots of b's cells snaps[snap_begin, snap_begin + snap_count).
// No op reads a cell that the same fill writes (those reads go through the
// snapshots), and every kernel of the step writes only the cells of its own
// block.  So a fill can run inside the kernel that consumes the field, each
// CTA gathering its own block's ghost cells first, provided that the kernel
// before it (which writes no cell the gathers read) saved the snapshots:
// each of its CTAs saves its own block's, after its own writes.
struct FillPass {
  GhostSeg seg[kMaxSeg];
  int nseg;             // 0: no fill
  int rows;             // variables over the segments
  int tile_seg;         // segment mirrored in the consuming kernel's shared memory (-1: none)
  double *snapbuf;      // [nseg][nsnaps][8]
};
struct FillFuse {
  const GhostOp *ops;
  const GhostSnap *snaps;
  int nsnaps;           // snapshot rows per segment in a buffer
  FillPass apply;       // the fill this kernel consumes: gathered into the CTA's block first
  FillPass save;        // the next fill: the CTA's block's snapshots, saved last
};

__device__ __forceinline__ GhostSeg pass_seg(const FillPass &p, int row, int &q, int &k) {
  GhostSeg s = p.seg[0];
  q = 0;
  k = row;
  if (p.nseg > 1 && k >= s.nv) { k -= s.nv; s = p.seg[1]; q = 1; }
  if (p.nseg > 2 && k >= s.nv) { k -= s.nv; s = p.seg[2]; q = 2; }
  return s;
}

// the gathers of the fill `f.apply` into the ghost cells of task t's block
// (variable-major, so that consecutive threads take consecutive ops); the
// caller synchronises the CTA afterwards
template <int N, typename TileT>
__device__ __forceinline__ void fill_apply_task(const FillFuse &f, const LeafTask &t, int tid, int nthr,
                                                TileT *tile) {
  const int n = t.op_count;
  const int total = n * f.apply.rows;
  for (int e = tid; e < total; e += nthr) {
    const int row = e / n;
    const GhostOp op = f.ops[t.op_begin + (e - row * n)];
    int q, k;
    const GhostSeg s = pass_seg(f.apply, row, q, k);
    const double *snap = f.apply.snapbuf + static_cast<size_t>(q) * f.nsnaps * 8;
    TileT *tl = q == f.apply.tile_seg ? tile : nullptr;
    if (s.f32) ghost_apply_one<N, float>(s, op, k, snap, reinterpret_cast<float *>(tl));
    else ghost_apply_one<N, double>(s, op, k, snap, reinterpret_cast<double *>(tl));
  }
}

// The first gather of a thread, loaded ahead (while the fused stage
// kernel's bulk copy is in flight) and stored by fill_apply_task_after; the
// values are held as double (exact for float fields).
struct FillPre {
  GhostOp op;
  double v0, v1;
  int row;
  bool on;
};

template <int N>
__device__ __forceinline__ FillPre fill_prefetch(const FillFuse &f, const LeafTask &t, int tid) {
  FillPre p{};
  const int n = t.op_count;
  p.on = f.apply.nseg != 0 && tid < n * f.apply.rows;
  if (!p.on) return p;
  p.row = tid / n;
  p.op = f.ops[t.op_begin + (tid - p.row * n)];
  int q, k;
  const GhostSeg s = pass_seg(f.apply, p.row, q, k);
  const double *snap = f.apply.snapbuf + static_cast<size_t>(q) * f.nsnaps * 8;
  if (s.f32) {
    float a = 0.f, b = 0.f;
    ghost_gather<N, float>(s, p.op, k, snap, a, b);
    p.v0 = a;
    p.v1 = b;
  } else {
    ghost_gather<N, double>(s, p.op, k, snap, p.v0, p.v1);
  }
  return p;
}

// fill_apply_task with the thread's first gather already loaded in `p`
template <int N, typename TileT>
__device__ __forceinline__ void fill_apply_task_after(const FillFuse &f, const LeafTask &t, int tid, int nthr,
                                                      TileT *tile, const FillPre &p) {
  if (p.on) {
    int q, k;
    const GhostSeg s = pass_seg(f.apply, p.row, q, k);
    TileT *tl = q == f.apply.tile_seg ? tile : nullptr;
    if (s.f32)
      ghost_put<N, float>(s, p.op, k, static_cast<float>(p.v0), static_cast<float>(p.v1),
                          reinterpret_cast<float *>(tl));
    else
      ghost_put<N, double>(s, p.op, k, p.v0, p.v1, reinterpret_cast<double *>(tl));
  }
  const int n = t.op_count;
  const int total = n * f.apply.rows;
  for (int e = tid + nthr; e < total; e += nthr) {
    const int row = e / n;
    const GhostOp op = f.ops[t.op_begin + (e - row * n)];
    int q, k;
    const GhostSeg s = pass_seg(f.apply, row, q, k);
    const double *snap = f.apply.snapbuf + static_cast<size_t>(q) * f.nsnaps * 8;
    TileT *tl = q == f.apply.tile_seg ? tile : nullptr;
    if (s.f32) ghost_apply_one<N, float>(s, op, k, snap, reinterpret_cast<float *>(tl));
    else ghost_apply_one<N, double>(s, op, k, snap, reinterpret_cast<double *>(tl));
  }
}

__device__ __forceinline__ void snap_one(const FillFuse &f, int NN, const GhostSnap &sn, int r, int row) {
  int q, k;
  const GhostSeg s = pass_seg(f.save, row, q, k);
  const size_t at = (static_cast<size_t>(sn.slot) * s.nv + k) * NN + sn.pos;
  f.save.snapbuf[(static_cast<size_t>(q) * f.nsnaps + r) * 8 + k] =
      s.f32 ? static_cast<double>(static_cast<const float *>(s.field)[at]) : static_cast<const double *>(s.field)[at];
}

// the snapshots of the next fill (`f.save`) that lie in task t's block; the
// caller synchronises the CTA before, after its own writes to the fields
template <int N>
__device__ __forceinline__ void fill_save_task(const FillFuse &f, const LeafTask &t, int tid, int nthr) {
  const int n = t.snap_count;
  const int total = n * f.save.rows;
  for (int e = tid; e < total; e += nthr) {
    const int row = e / n;
    const int r = t.snap_begin + (e - row * n);
    snap_one(f, N * N, f.snaps[r], r, row);
  }
}

// every snapshot of the next fill, from any thread of the grid: for a
// kernel that writes none of the saved fields
template <int N>
__device__ __forceinline__ void fill_save_all(const FillFuse &f, size_t gtid, size_t gsize) {
  const size_t total = static_cast<size_t>(f.nsnaps) * f.save.rows;
  for (size_t e = gtid; e < total; e += gsize) {
    const int row = static_cast<int>(e / f.nsnaps);
    const int r = static_cast<int>(e - static_cast<size_t>(row) * f.nsnaps);
    const GhostSnap sn = f.snaps[r];
    if (sn.slot >= 0) snap_one(f, N * N, sn, r, row);
  }
}

}  // namespace amr
