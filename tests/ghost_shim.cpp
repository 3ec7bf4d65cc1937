// Test infrastructure: runs the product's host ghost-fill compiler
// (amr2d_mhd_gb300/csrc/ghost_compile.cpp) on a given quadtree and applies the
// compiled gathers on the CPU the way k_ghost_snap / k_ghost_apply do, so the
// compiler can be checked against the oracle's sequential fill without a GPU.
#include <cstring>
#include <string>
#include <vector>

#include "ghost_compile.hpp"

extern "C" int ghost_shim_apply(int last_active, const int *lp, const int *icoord, const unsigned char *leafs,
                                int maxlevs, int nrx, int nry, int periodic, int ng, int kind, int nv,
                                double *field, int *n_ops, int *n_snaps) {
  using namespace amr;
  TreeShape s{16, 16, ng, maxlevs, nrx, nry, periodic != 0};
  Tree t(s);
  if (last_active > t.maxblocks()) return -1;
  t.lastActive = last_active;
  for (int b = 0; b < last_active; b++) {
    for (int q = 0; q < 8; q++) t.lp[b][q] = lp[8 * b + q];
    t.icoord[b] = {icoord[2 * b], icoord[2 * b + 1]};
    t.leafs[b] = leafs[b];
  }
  std::vector<Bound> bounds;
  t.locate_bounds(bounds);
  const int n = 16 + 2 * ng, nn = n * n;
  std::vector<int> slot(last_active);
  for (int b = 0; b < last_active; b++) slot[b] = b;
  GhostCompiler gc(n, ng);
  GhostProgram p;
  gc.compile(t, bounds, static_cast<FillKind>(kind), nv, slot.data(), 0, p);
  std::vector<double> snap(p.snaps.size() * 8);
  for (size_t i = 0; i < p.snaps.size(); i++)
    for (int k = p.snaps[i].k0; k < p.snaps[i].k1; k++)
      snap[i * 8 + k] = field[(static_cast<size_t>(p.snaps[i].slot) * nv + k) * nn + p.snaps[i].pos];
  // gathers read only pre-fill values: evaluate all, then write
  std::vector<double> out;
  for (const GhostOp &op : p.ops)
    for (int k = op.k0; k < op.k1; k++) {
      const double *src = field + (static_cast<size_t>(op.src_slot) * nv + k) * nn + op.src_pos;
      double v;
      if (op.type == GOP_COPY) v = src[0];
      else if (op.type == GOP_SNAP) v = snap[static_cast<size_t>(op.src_slot) * 8 + k];
      else if (op.type == GOP_AVG4) { double a = 0.; a += src[0]; a += src[n]; a += src[1]; a += src[1 + n]; v = 0.25 * a; }
      else if (op.type == GOP_AVGJ) { double a = 0.; a += src[0]; a += src[n]; v = 0.5 * a; }
      else if (op.type == GOP_AVGI) { double a = 0.; a += src[0]; a += src[1]; v = 0.5 * a; }
      else {
        const int nc = op.type == GOP_SAVG4 ? 4 : 2;
        double a = 0.;
        for (int c = 0; c < nc; c++) a += snap[(static_cast<size_t>(op.src_slot) + c) * 8 + k];
        v = (op.type == GOP_SAVG4 ? 0.25 : 0.5) * a;
      }
      out.push_back(v);
    }
  size_t q = 0;
  for (const GhostOp &op : p.ops)
    for (int k = op.k0; k < op.k1; k++)
      field[(static_cast<size_t>(op.dst_slot) * nv + k) * nn + op.dst_pos] = out[q++];
  *n_ops = static_cast<int>(p.ops.size());
  *n_snaps = static_cast<int>(p.snaps.size());
  return 0;
}

// the product's Tree::admesh on a given tree and per-block criterion; writes
// the new tree back and returns the number of refine and coarsen operations
extern "C" int tree_shim_admesh(int *last_active, int *lp, int *icoord, unsigned char *leafs, int *nbleafs,
                                int maxlevs, int nrx, int nry, int periodic, int ng, const double *grad,
                                int cap, int *n_ref, int *n_crs) {
  using namespace amr;
  TreeShape s{16, 16, ng, maxlevs, nrx, nry, periodic != 0};
  Tree t(s);
  t.lastActive = *last_active;
  t.nbleafs = *nbleafs;
  for (int b = 0; b < t.lastActive; b++) {
    for (int q = 0; q < 8; q++) t.lp[b][q] = lp[8 * b + q];
    t.icoord[b] = {icoord[2 * b], icoord[2 * b + 1]};
    t.leafs[b] = leafs[b];
  }
  std::vector<double> g(grad, grad + t.lastActive);
  AdmeshPlan plan;
  std::string err;
  if (!t.admesh(g, plan, err)) return -1;
  if (t.lastActive > cap) return -2;
  *last_active = t.lastActive;
  *nbleafs = t.nbleafs;
  for (int b = 0; b < t.lastActive; b++) {
    for (int q = 0; q < 8; q++) lp[8 * b + q] = t.lp[b][q];
    icoord[2 * b] = t.icoord[b][0];
    icoord[2 * b + 1] = t.icoord[b][1];
    leafs[b] = t.leafs[b];
  }
  *n_ref = static_cast<int>(plan.refine.size());
  *n_crs = static_cast<int>(plan.coarsen.size());
  return 0;
}
