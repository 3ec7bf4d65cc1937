// Host-side quadtree of one AMR instance: the metadata the reference keeps in
// meshblock::lp / icoord / leafs / iref / icoarse (defs.hpp:52-62), the
// boundary list of locate_bounds.cpp, and the tree half of admesh.cpp.  The
// field data never comes here; admesh returns the refine / coarsen operations
// for the device to apply.
#pragma once

#include <array>
#include <cstdint>
#include <string>
#include <vector>

namespace amr {

// innerbounds entry (locate_bounds.cpp:14-30): source block, neighbour block,
// direction code (1/4/7/10 same level, 2/5/8/11 finer neighbour, -1..-4 box)
struct Bound {
  int src, dst, code;
};

struct TreeShape {
  int ni, nj;      // interior cells per block
  int ng;          // ghost layers
  int maxlevs;
  int nrx, nry;    // root blocks
  bool periodic;
};

struct AdmeshPlan {
  std::vector<std::array<int, 5>> refine;   // dad, son1..son4 (block IDs)
  std::vector<std::array<int, 5>> coarsen;  // dad, son1..son4
};

class Tree {
 public:
  explicit Tree(const TreeShape &s);

  int maxblocks() const { return maxblocks_; }
  int nroots() const { return shape_.nrx * shape_.nry; }
  const TreeShape &shape() const { return shape_; }

  // basegrid.cpp:4-89, generalised from 2x2 to nrx x nry roots (row-major IDs)
  void basegrid();
  // locate_bounds.cpp:35-208
  void locate_bounds(std::vector<Bound> &out) const;
  std::vector<int> leaves() const;
  // The structure every tree admesh builds: IDs in range, father / son and
  // sibling links consistent, the active tree 2:1 balanced.  A tree handed
  // in from outside must pass before its IDs reach ghost programs or
  // refine / coarsen operations.  Returns false with `err` otherwise.
  bool check(std::string &err) const;

  // admesh.cpp:17-102.  grad[nb] is, for each leaf, the largest relative
  // jump of criteria.cpp:11-29 over the block (only leaves are read).
  // Applies refine / coarsen to the tree and lists them in `plan`.
  // Returns false (with `err`) when the block budget is exceeded.
  bool admesh(const std::vector<double> &grad, AdmeshPlan &plan, std::string &err);
  // admesh.cpp:17-102 with the caller's marks in place of criteria.cpp's:
  // mark_ref[nb] / mark_crs[nb] are read for leaves only; a refine mark on
  // the finest level is dropped and cancels a coarsen mark, as in
  // criteria.cpp:31-43.  The neighbour rules and the operations are admesh's.
  bool admesh_marked(const uint8_t *mark_ref, const uint8_t *mark_crs, AdmeshPlan &plan, std::string &err);

  std::vector<std::array<int, 8>> lp;      // level, father, first son, sibling, L, R, D, U
  std::vector<std::array<int, 2>> icoord;  // block origin in cells of its own level
  std::vector<uint8_t> leafs, iref, icoarse;
  int lastActive = 0;
  int nbleafs = 0;   // the reference's counter (refine adds 4, coarsen removes 3)
  uint64_t version = 0;  // bumped whenever the tree changes

 private:
  // critneighup / refine / critneighdown / coarsen on iref and icoarse
  bool apply_marks(AdmeshPlan &plan, std::string &err);
  void updatelpup(int nb, const int *s);
  void updatelpdown(int dad, const int *s);
  TreeShape shape_;
  int maxblocks_;
};

}  // namespace amr
