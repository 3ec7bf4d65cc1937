// Test infrastructure: runs the product's host ghost-fill compiler
// (amr2d_mhd_gb300/csrc/ghost_compile.cpp) on a given quadtree and applies the
// compiled gathers on the CPU the way k_ghost_snap / k_ghost_apply do, so the
// compiler can be checked against the oracle's sequential fill without a GPU.
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "ghost_compile.hpp"
#include "host_par.hpp"

static int g_last_by_block = -1;
// 1 if the last compiled program had every destination and snapshot in a leaf
extern "C" int ghost_shim_last_by_block() { return g_last_by_block; }

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
  gc.compile(t, bounds, slot.data(), p);
  // grouping by block: block b's ops write only b, its snapshots read only b
  if (p.op_start.size() != static_cast<size_t>(last_active) + 1 ||
      p.snap_start.size() != static_cast<size_t>(last_active) + 1 || p.op_start[0] != 0 || p.snap_start[0] != 0 ||
      p.op_start[last_active] != static_cast<int>(p.ops.size()) ||
      p.snap_start[last_active] != static_cast<int>(p.snaps.size()))
    return -3;
  bool leaves_only = true;
  for (int b = 0; b < last_active; b++) {
    if (p.op_start[b + 1] < p.op_start[b] || p.snap_start[b + 1] < p.snap_start[b]) return -3;
    for (int o = p.op_start[b]; o < p.op_start[b + 1]; o++)
      if (p.ops[o].dst_slot != slot[b]) return -3;
    for (int r = p.snap_start[b]; r < p.snap_start[b + 1]; r++)
      if (p.snaps[r].slot != slot[b]) return -3;
    if ((p.op_start[b + 1] > p.op_start[b] || p.snap_start[b + 1] > p.snap_start[b]) && !t.leafs[b])
      leaves_only = false;
  }
  if (leaves_only != p.by_block) return -3;
  g_last_by_block = p.by_block ? 1 : 0;
  std::vector<double> snap(p.snaps.size() * 8);
  for (size_t i = 0; i < p.snaps.size(); i++)
    for (int k = 0; k < nv; k++)
      snap[i * 8 + k] = field[(static_cast<size_t>(p.snaps[i].slot) * nv + k) * nn + p.snaps[i].pos];
  // the fine-to-coarse value per kind of field (boundary.cpp:48,
  // boundaryfc.cpp:48, boundaryec.cpp:46)
  auto fine = [&](int k, double a00, double a01, double a10, double a11) {
    double v = 0.;
    if (kind == FILL_CC) { v += a00; v += a01; v += a10; v += a11; return 0.25 * v; }
    if (kind == FILL_FC) { v += a00; v += k == 0 ? a01 : a10; return 0.5 * v; }
    return a00;
  };
  // gathers read only pre-fill values: evaluate all, then write
  std::vector<double> out;
  for (const GhostOp &op : p.ops)
    for (int k = 0; k < nv; k++) {
      const double *src = field + (static_cast<size_t>(op.src_slot) * nv + k) * nn + op.src_pos;
      const double *r = snap.data() + static_cast<size_t>(op.src_slot) * 8 + k;
      double v;
      if (op.type == GOP_COPY || op.type == GOP_COPY2) v = src[0];
      else if (op.type == GOP_SNAP) v = r[0];
      else if (op.type == GOP_FINE) v = fine(k, src[0], src[n], src[1], src[1 + n]);
      else v = fine(k, r[0], r[8], r[16], r[24]);
      out.push_back(v);
      if (op.type == GOP_COPY2) {
        if ((op.dst_pos & 1) || (op.src_pos & 1)) return -2;  // a pair must be aligned
        out.push_back(src[1]);
      }
    }
  size_t q = 0;
  for (const GhostOp &op : p.ops)
    for (int k = 0; k < nv; k++) {
      field[(static_cast<size_t>(op.dst_slot) * nv + k) * nn + op.dst_pos] = out[q++];
      if (op.type == GOP_COPY2) field[(static_cast<size_t>(op.dst_slot) * nv + k) * nn + op.dst_pos + 1] = out[q++];
    }
  *n_ops = static_cast<int>(p.ops.size());
  *n_snaps = static_cast<int>(p.snaps.size());
  return 0;
}

// The fill as the fused kernels run it: every block's snapshots saved first
// (by the kernel before), then each block's gathers applied in place, one
// block after another in a shuffled order (the CTAs of the consuming
// kernel), each write visible at once.  The result equals the sequential
// walk only if no gather reads a cell that another block's gathers write.
extern "C" int ghost_shim_apply_fused(int last_active, const int *lp, const int *icoord, const unsigned char *leafs,
                                      int maxlevs, int nrx, int nry, int periodic, int ng, int kind, int nv,
                                      double *field, unsigned seed) {
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
  gc.compile(t, bounds, slot.data(), p);
  if (!p.by_block) return -4;
  std::vector<int> order(last_active);
  for (int b = 0; b < last_active; b++) order[b] = b;
  auto shuffle = [&]() {  // Fisher-Yates with a small LCG (deterministic per seed)
    for (int b = last_active - 1; b > 0; b--) {
      seed = seed * 1664525u + 1013904223u;
      std::swap(order[b], order[(seed >> 8) % static_cast<unsigned>(b + 1)]);
    }
  };
  std::vector<double> snap(p.snaps.size() * 8);
  shuffle();
  for (int b : order)
    for (int r = p.snap_start[b]; r < p.snap_start[b + 1]; r++)
      for (int k = 0; k < nv; k++)
        snap[static_cast<size_t>(r) * 8 + k] =
            field[(static_cast<size_t>(p.snaps[r].slot) * nv + k) * nn + p.snaps[r].pos];
  auto fine = [&](int k, double a00, double a01, double a10, double a11) {
    double v = 0.;
    if (kind == FILL_CC) { v += a00; v += a01; v += a10; v += a11; return 0.25 * v; }
    if (kind == FILL_FC) { v += a00; v += k == 0 ? a01 : a10; return 0.5 * v; }
    return a00;
  };
  shuffle();
  for (int b : order)
    for (int o = p.op_start[b]; o < p.op_start[b + 1]; o++) {
      const GhostOp &op = p.ops[o];
      for (int k = 0; k < nv; k++) {
        const double *src = field + (static_cast<size_t>(op.src_slot) * nv + k) * nn + op.src_pos;
        const double *r = snap.data() + static_cast<size_t>(op.src_slot) * 8 + k;
        double *dst = field + (static_cast<size_t>(op.dst_slot) * nv + k) * nn + op.dst_pos;
        if (op.type == GOP_COPY2) {
          const double v0 = src[0], v1 = src[1];
          dst[0] = v0;
          dst[1] = v1;
        } else if (op.type == GOP_COPY) {
          dst[0] = src[0];
        } else if (op.type == GOP_SNAP) {
          dst[0] = r[0];
        } else if (op.type == GOP_FINE) {
          dst[0] = fine(k, src[0], src[n], src[1], src[1 + n]);
        } else {
          dst[0] = fine(k, r[0], r[8], r[16], r[24]);
        }
      }
    }
  return 0;
}

// the product's Tree::admesh on a given tree and per-block criterion (or,
// with grad NULL, Tree::admesh_marked on the marks mref / mcrs); writes the
// new tree back and returns the number of refine and coarsen operations
extern "C" int tree_shim_admesh(int *last_active, int *lp, int *icoord, unsigned char *leafs, int *nbleafs,
                                int maxlevs, int nrx, int nry, int periodic, int ng, const double *grad,
                                int cap, int *n_ref, int *n_crs, const unsigned char *mref,
                                const unsigned char *mcrs) {
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
  AdmeshPlan plan;
  std::string err;
  if (grad) {
    std::vector<double> g(grad, grad + t.lastActive);
    if (!t.admesh(g, plan, err)) return -1;
  } else if (!t.admesh_marked(mref, mcrs, plan, err)) {
    return -1;
  }
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

// Tree::check on a given tree: 0 when it passes, 1 (message in err) when not
extern "C" int tree_shim_check(int last_active, const int *lp, const int *icoord, const unsigned char *leafs,
                               int maxlevs, int nrx, int nry, int periodic, int ng, char *err, int errlen) {
  using namespace amr;
  TreeShape s{16, 16, ng, maxlevs, nrx, nry, periodic != 0};
  Tree t(s);
  if (last_active > t.maxblocks()) return 2;
  t.lastActive = last_active;
  for (int b = 0; b < last_active; b++) {
    for (int q = 0; q < 8; q++) t.lp[b][q] = lp[8 * b + q];
    t.icoord[b] = {icoord[2 * b], icoord[2 * b + 1]};
    t.leafs[b] = leafs[b];
  }
  std::string e;
  if (t.check(e)) return 0;
  std::snprintf(err, static_cast<size_t>(errlen), "%s", e.c_str());
  return 1;
}

// The engine's host thread pool: `rounds` parallel loops of n items on up to
// `threads` threads (the calling one included); each item adds its index to a
// per-round sum.  Returns the number of rounds whose sum is wrong.
extern "C" int host_pool_shim(int rounds, int n, int threads) {
  amr::HostPool pool;
  int bad = 0;
  for (int r = 0; r < rounds; r++) {
    std::vector<long long> part(static_cast<size_t>(threads), 0);
    const std::string err = amr::parallel_items(pool, static_cast<size_t>(n), static_cast<size_t>(threads),
                                                [&](size_t w, size_t q) { part[w] += static_cast<long long>(q) + r; });
    long long sum = 0;
    for (long long v : part) sum += v;
    const long long want = static_cast<long long>(n) * (n - 1) / 2 + static_cast<long long>(n) * r;
    bad += (sum != want || !err.empty()) ? 1 : 0;
  }
  return bad;
}
