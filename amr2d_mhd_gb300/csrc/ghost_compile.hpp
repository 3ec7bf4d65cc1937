// Compiles the reference's sequential ghost fills into order-free gather lists.
//
// boundary.cpp / boundaryfc.cpp / boundaryec.cpp walk the innerbounds list in
// order and copy or average cells between blocks; later copies can read ghost
// cells that earlier ones wrote (full-height column copies include the source's
// ghost rows, injections read the coarse block's ghost ring), so the result
// depends on the order.  The compiler replays that order symbolically on the
// host: every ghost cell ends up as "the pre-fill value of cell X" or "the
// average of interior cells of block B".  The GPU then applies all gathers at
// once; pre-fill values of cells the same fill overwrites are saved first
// (GhostSnap).  The result is bit-identical to the sequential walk.
#pragma once

#include <cstdint>
#include <vector>

#include "amr_common.h"
#include "tree.hpp"

namespace amr {

// cell centred (boundary.cpp), face centred (boundaryfc.cpp), edge centred
// (boundaryec.cpp)
enum FillKind { FILL_CC = 0, FILL_FC = 1, FILL_EC = 2 };

// The program of one instance, grouped by block: the ops that write block
// b's ghost cells are ops[op_start[b], op_start[b+1]) and the snapshots of
// b's cells snaps[snap_start[b], snap_start[b+1]).  `by_block` is false when
// a destination or a snapshot lies in a block that is not a leaf (the fill
// can then only run as a launch of its own).
struct GhostProgram {
  std::vector<GhostOp> ops;
  std::vector<GhostSnap> snaps;
  std::vector<int> op_start, snap_start;
  bool by_block = false;
  void clear() {
    ops.clear();
    snaps.clear();
    op_start.clear();
    snap_start.clear();
    by_block = false;
  }
};

class GhostCompiler {
 public:
  // n = block edge with ghosts, ng = ghost layers
  GhostCompiler(int n, int ng) : n_(n), ng_(ng) {}
  // Writes the gathers of one instance's ghost fill (any kind of field) to
  // `out` (cleared first), grouped by block.  `slot` maps block IDs to
  // physical device slots.
  void compile(const Tree &t, const std::vector<Bound> &bounds, const int *slot, GhostProgram &out);

 private:
  struct Desc {
    int blk;        // block ID (logical)
    int16_t pos;    // j * n + i
    uint8_t type;   // GOP_COPY: pre-fill value of (blk,pos); GOP_FINE: 2x2 patch at (blk,pos)
  };
  Desc get(int blk, int pos) const;
  void set(int blk, int pos, const Desc &d);
  void run_sequence(const Tree &t, const std::vector<Bound> &bounds);
  bool overwritten(int blk, int pos) const;

  int n_, ng_;
  int nn_ = 0;
  uint32_t gen_ = 0;
  std::vector<uint32_t> stamp_;
  std::vector<Desc> cur_;
  std::vector<int> touched_;
  std::vector<uint32_t> snap_stamp_;
  std::vector<int> snap_row_;
  std::vector<uint32_t> emit_stamp_;  // cell already written by an emitted op
  // grouping by block after the emission (kept apart from the replay and
  // emission loops, whose speed depends on their code staying small)
  void group_by_block(const Tree &t, const int *slot, GhostProgram &out);
  std::vector<int> blk_of_slot_;      // inverse of `slot` for this instance's blocks
  std::vector<int> count_;
  std::vector<GhostOp> ops_tmp_;
  std::vector<GhostSnap> snaps_tmp_;
  std::vector<int> snap_perm_;        // emission row -> grouped row
};

}  // namespace amr
