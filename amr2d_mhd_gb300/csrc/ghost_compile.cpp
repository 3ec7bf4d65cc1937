// Symbolic replay of boundary.cpp / boundaryfc.cpp / boundaryec.cpp /
// extboundary.cpp; see ghost_compile.hpp.
#include "ghost_compile.hpp"

#include <algorithm>
#include <stdexcept>
#include <unordered_map>

namespace amr {

GhostCompiler::Desc GhostCompiler::get(int blk, int pos) const {
  const size_t idx = static_cast<size_t>(blk) * nn_ + pos;
  if (stamp_[idx] == gen_) return cur_[idx];
  return Desc{blk, static_cast<int16_t>(pos), 0};
}

void GhostCompiler::set(int blk, int pos, const Desc &d) {
  const size_t idx = static_cast<size_t>(blk) * nn_ + pos;
  if (stamp_[idx] != gen_) {
    stamp_[idx] = gen_;
    touched_.push_back(static_cast<int>(idx));
  }
  cur_[idx] = d;
}

// One pass over the innerbounds list.  The index arithmetic is that of
// boundary.cpp, identical in the three files; the fine-to-coarse value is kept
// symbolic (GOP_FINE) and made concrete per kind of field by the kernel.
void GhostCompiler::run_sequence(const Tree &t, const std::vector<Bound> &bounds) {
  const int n = n_, ng = ng_, nx = n, ny = n;
  const int nxmin = ng, nxmax = n - 1 - ng, nymin = ng, nymax = n - 1 - ng;
  const int nxminb = nxmin - 1, nxmaxb = nxmax + 1, nyminb = nymin - 1, nymaxb = nymax + 1;
  const int nxp1 = nxmaxb, nyp1 = nymaxb;
  const int nx2 = (n - 1) / 2, ny2 = (n - 1) / 2;
  const auto &lp = t.lp;
  const auto &leafs = t.leafs;
  auto P = [n](int i, int j) { return j * n + i; };
  auto interior = [&](int i, int j) { return i >= nxmin && i <= nxmax && j >= nymin && j <= nymax; };
  // plain copy of one cell (all three files)
  auto C = [&](int db, int di, int dj, int sb, int si, int sj) {
    set(db, P(di, dj), get(sb, P(si, sj)));
  };
  // fine-to-coarse value with lower-left source cell (i1, j1).  With 4 ghost
  // layers the reference's left / bottom stencils reach one ghost column /
  // row of the fine block (boundary.cpp:43 and :227 give 2i+13 where 2i+12 is
  // meant); such a cell must still hold its pre-fill value here, and
  // compile() saves it first if the fill overwrites it later.
  auto Fv = [&](int db, int di, int dj, int sb, int i1, int j1) {
    for (int i = i1; i <= i1 + 1; i++)
      for (int j = j1; j <= j1 + 1; j++) {
        if (interior(i, j)) continue;
        const Desc d = get(sb, P(i, j));
        if (!(d.type == GOP_COPY && d.blk == sb && d.pos == P(i, j)))
          throw std::logic_error("ghost compile: fine average of an already filled ghost cell");
      }
    set(db, P(di, dj), Desc{sb, static_cast<int16_t>(P(i1, j1)), GOP_FINE});
  };

  for (const Bound &b : bounds) {
    const int nbs = b.src;
    int n1, n2, n3, n4, ii, jj;
    switch (b.code) {
      case 1:  // left, same level (boundary.cpp:17-35)
        n1 = b.dst;
        for (int j = 0; j < ny; j++) {
          ii = nxmax - (ng - 1);
          for (int i = 0; i < ng; i++, ii++) C(nbs, i, j, n1, ii, j);
          ii = nxmin;
          for (int i = nxp1; i < nx; i++, ii++) C(n1, i, j, nbs, ii, j);
        }
        break;
      case 2:  // left, finer neighbour (boundary.cpp:36-107)
        n1 = b.dst;
        n2 = n1 + 2;
        for (int j = nymin; j <= ny2; j++) {
          const int ny2j = ny2 + j - 1 - (ng - 2);
          for (int i = 0; i < ng; i++) {
            const int i1 = 2 * (i - ng / 2) - ng / 2 + nxmax, j1 = 2 * j - nymin;
            Fv(nbs, i, j, n1, i1, j1);
            Fv(nbs, i, ny2j, n2, i1, j1);
          }
        }
        n3 = lp[lp[n1][1]][6];
        if (n3 != -1) {
          if (leafs[n3]) {
            for (int i = 0; i < ng; i++)
              for (int j = 0; j < ng; j++) C(nbs, i, j, n3, nxmax - ng + (i + 1), nymax - ng + (j + 1));
          } else {
            n3 = lp[n3][2] + 3;
            if (leafs[n3])
              for (int i = 0; i < ng; i++)
                for (int j = 0; j < ng; j++)
                  Fv(nbs, i, j, n3, nxmax - ng * 2 + 2 * i + 1, nymax - ng * 2 + 2 * j + 1);
          }
        }
        n4 = lp[lp[n2][1]][7];
        if (n4 != -1) {
          if (leafs[n4]) {
            for (int i = 0; i < ng; i++)
              for (int j = 0; j < ng; j++)
                C(nbs, i, ny - 1 - j, n4, nxmax - ng + (i + 1), nymin + ng - (j + 1));
          } else {
            n4 = lp[n4][2] + 1;
            if (leafs[n4])
              for (int i = 0; i < ng; i++)
                for (int j = 0; j < ng; j++)
                  Fv(nbs, i, ny - 1 - j, n4, nxmax - ng * 2 + 2 * i + 1, nymin + ng * 2 - 2 * (j + 1));
          }
        }
        for (int i = 1; i <= ng; i++)
          for (int j = 0; j < ny; j++) {
            C(n1, i + nxmax, j, nbs, (i + 2 * ng - 1) / 2, (j + ng) / 2);
            C(n2, i + nxmax, j, nbs, (i + 2 * ng - 1) / 2, (j - ng + 2) / 2 + ny2);
          }
        break;
      case 4:  // right, same level (boundary.cpp:109-127)
        n1 = b.dst;
        for (int j = 0; j < ny; j++) {
          ii = nxmin;
          for (int i = nxp1; i < nx; i++, ii++) C(nbs, i, j, n1, ii, j);
          ii = nxmax - (ng - 1);
          for (int i = 0; i < ng; i++, ii++) C(n1, i, j, nbs, ii, j);
        }
        break;
      case 5:  // right, finer neighbour (boundary.cpp:128-197)
        n1 = b.dst;
        n2 = n1 + 2;
        for (int i = nxp1; i < nx; i++)
          for (int j = nymin; j <= ny2; j++) {
            const int i1 = 2 * (i - nxmax + (ng / 2 - 1)), j1 = 2 * j - nymin;
            const int ny2j = ny2 + j - 1 - (ng - 2);
            Fv(nbs, i, j, n1, i1, j1);
            Fv(nbs, i, ny2j, n2, i1, j1);
          }
        n3 = lp[lp[n1][1]][6];
        if (n3 != -1) {
          if (leafs[n3]) {
            for (int i = nxmaxb; i < nx; i++)
              for (int j = 0; j < ng; j++) C(nbs, i, j, n3, nxminb + (i - nxmax), nymax - ng + (j + 1));
          } else {
            n3 = lp[n3][2] + 2;
            if (leafs[n3])
              for (int i = nxmaxb; i < nx; i++)
                for (int j = 0; j < ng; j++)
                  Fv(nbs, i, j, n3, nxminb + 2 * (i - nxmax) - 1, nymax - ng * 2 + 2 * j + 1);
          }
        }
        n4 = lp[lp[n2][1]][7];
        if (n4 != -1) {
          if (leafs[n4]) {
            for (int i = nxmaxb; i < nx; i++)
              for (int j = 0; j < ng; j++)
                C(nbs, i, ny - 1 - j, n4, nxminb + (i - nxmax), nymin + ng - (j + 1));
          } else {
            n4 = lp[n4][2];
            if (leafs[n4])
              for (int i = nxmaxb; i < nx; i++)
                for (int j = 0; j < ng; j++)
                  Fv(nbs, i, ny - 1 - j, n4, nxminb + 2 * (i - nxmax) - 1, nymin + ng * 2 - 2 * (j + 1));
          }
        }
        for (int i = 1; i <= ng; i++)
          for (int j = 0; j < ny; j++) {
            C(n1, i - 1, j, nbs, (i + 1) / 2 + nxmax - ng / 2, (j + ng) / 2);
            C(n2, i - 1, j, nbs, (i + 1) / 2 + nxmax - ng / 2, (j - ng + 2) / 2 + ny2);
          }
        break;
      case 7:  // bottom, same level (boundary.cpp:199-217)
        n1 = b.dst;
        for (int i = 0; i < nx; i++) {
          jj = nymax - (ng - 1);
          for (int j = 0; j < ng; j++, jj++) C(nbs, i, j, n1, i, jj);
          jj = nymin;
          for (int j = nyp1; j < ny; j++, jj++) C(n1, i, j, nbs, i, jj);
        }
        break;
      case 8:  // bottom, finer neighbour (boundary.cpp:218-287)
        n1 = b.dst;
        n2 = n1 + 1;
        for (int i = nxmin; i <= nx2; i++) {
          const int nx2i = nx2 + i - 1 - (ng - 2);
          for (int j = 0; j < ng; j++) {
            const int i1 = 2 * i - nxmin, j1 = 2 * (j - ng / 2) - ng / 2 + nymax;
            Fv(nbs, i, j, n1, i1, j1);
            Fv(nbs, nx2i, j, n2, i1, j1);
          }
        }
        n3 = lp[lp[n1][1]][4];
        if (n3 != -1) {
          if (leafs[n3]) {
            for (int i = 0; i < ng; i++)
              for (int j = 0; j < ng; j++) C(nbs, i, j, n3, nxmax - ng + (i + 1), nymax - ng + (j + 1));
          } else {
            n3 = lp[n3][2] + 3;
            if (leafs[n3])
              for (int i = 0; i < ng; i++)
                for (int j = 0; j < ng; j++)
                  Fv(nbs, i, j, n3, nxmax - ng * 2 + 2 * i + 1, nymax - ng * 2 + 2 * j + 1);
          }
        }
        n4 = lp[lp[n2][1]][5];
        if (n4 != -1) {
          if (leafs[n4]) {
            for (int i = 0; i < ng; i++)
              for (int j = 0; j < ng; j++)
                C(nbs, nx - 1 - i, j, n4, nxmin + ng - (i + 1), nymax - ng + (j + 1));
          } else {
            n4 = lp[n4][2] + 2;
            if (leafs[n4])
              for (int i = 0; i < ng; i++)
                for (int j = 0; j < ng; j++)
                  Fv(nbs, nx - 1 - i, j, n4, nxmin + ng * 2 - 2 * (i + 1), nymax - ng * 2 + 2 * j + 1);
          }
        }
        for (int j = 1; j <= ng; j++)
          for (int i = 0; i < nx; i++) {
            C(n1, i, j + nymax, nbs, (i + ng) / 2, (j + 2 * ng - 1) / 2);
            C(n2, i, j + nymax, nbs, (i - ng + 2) / 2 + nx2, (j + 2 * ng - 1) / 2);
          }
        break;
      case 10:  // top, same level (boundary.cpp:289-307)
        n1 = b.dst;
        for (int i = 0; i < nx; i++) {
          jj = nymin;
          for (int j = nyp1; j < ny; j++, jj++) C(nbs, i, j, n1, i, jj);
          jj = nymax - (ng - 1);
          for (int j = 0; j < ng; j++, jj++) C(n1, i, j, nbs, i, jj);
        }
        break;
      case 11:  // top, finer neighbour (boundary.cpp:308-377)
        n1 = b.dst;
        n2 = n1 + 1;
        for (int i = nxmin; i <= nx2; i++)
          for (int j = nyp1; j < ny; j++) {
            const int i1 = 2 * i - nxmin, j1 = 2 * (j - nymax + (ng / 2 - 1));
            const int nx2i = nx2 + i - 1 - (ng - 2);
            Fv(nbs, i, j, n1, i1, j1);
            Fv(nbs, nx2i, j, n2, i1, j1);
          }
        n3 = lp[lp[n1][1]][4];
        if (n3 != -1) {
          if (leafs[n3]) {
            for (int i = 0; i < ng; i++)
              for (int j = nymaxb; j < ny; j++) C(nbs, i, j, n3, nxmax - ng + (i + 1), nyminb + (j - nymax));
          } else {
            n3 = lp[n3][2] + 1;
            if (leafs[n3])
              for (int i = 0; i < ng; i++)
                for (int j = nymaxb; j < ny; j++)
                  Fv(nbs, i, j, n3, nxmax - ng * 2 + 2 * i + 1, nyminb + 2 * (j - nymax) - 1);
          }
        }
        n4 = lp[lp[n2][1]][5];
        if (n4 != -1) {
          if (leafs[n4]) {
            for (int i = 0; i < ng; i++)
              for (int j = nymaxb; j < ny; j++)
                C(nbs, nx - 1 - i, j, n4, nxmin + ng - (i + 1), nyminb + (j - nymax));
          } else {
            n4 = lp[n4][2];
            if (leafs[n4])
              for (int i = nxmaxb; i < nx; i++)
                for (int j = nymaxb; j < ny; j++)
                  Fv(nbs, i, j, n4, nxminb + 2 * (i - nxmax) - 1, nyminb + 2 * (j - nymax) - 1);
          }
        }
        for (int j = 1; j <= ng; j++)
          for (int i = 0; i < nx; i++) {
            C(n1, i, j - 1, nbs, (i + ng) / 2, (j + 1) / 2 + nymax - ng / 2);
            C(n2, i, j - 1, nbs, (i - ng + 2) / 2 + nx2, (j + 1) / 2 + nymax - ng / 2);
          }
        break;
      default:
        break;
    }
  }
  // extboundary.cpp:5-61: mirror copy at the box, after all internal bounds
  for (const Bound &b : bounds) {
    const int nbs = b.src;
    int ii, jj;
    switch (b.code) {
      case -1:
        ii = nxmin + (ng - 1);
        for (int i = 0; i < ng; i++, ii--)
          for (int j = 0; j < ny; j++) C(nbs, i, j, nbs, ii, j);
        break;
      case -2:
        ii = nxmax;
        for (int i = nxp1; i < nx; i++, ii--)
          for (int j = 0; j < ny; j++) C(nbs, i, j, nbs, ii, j);
        break;
      case -3:
        jj = nymin + (ng - 1);
        for (int j = 0; j < ng; j++, jj--)
          for (int i = 0; i < nx; i++) C(nbs, i, j, nbs, i, jj);
        break;
      case -4:
        jj = nymax;
        for (int j = nyp1; j < ny; j++, jj--)
          for (int i = 0; i < nx; i++) C(nbs, i, j, nbs, i, jj);
        break;
      default:
        break;
    }
  }
}

bool GhostCompiler::overwritten(int blk, int pos) const {
  const size_t idx = static_cast<size_t>(blk) * nn_ + pos;
  if (stamp_[idx] != gen_) return false;
  const Desc &s = cur_[idx];
  return !(s.type == GOP_COPY && s.blk == blk && s.pos == pos);
}

void GhostCompiler::compile(const Tree &t, const std::vector<Bound> &bounds, const int *slot, GhostProgram &out) {
  nn_ = n_ * n_;
  const size_t need = static_cast<size_t>(t.lastActive) * nn_;
  if (stamp_.size() < need) {
    stamp_.resize(need, 0);
    cur_.resize(need);
    snap_stamp_.resize(need, 0);
    snap_row_.resize(need);
    emit_stamp_.resize(need, 0);
  }
  if (++gen_ == 0) {  // stamp wrap-around
    std::fill(stamp_.begin(), stamp_.end(), 0u);
    std::fill(snap_stamp_.begin(), snap_stamp_.end(), 0u);
    std::fill(emit_stamp_.begin(), emit_stamp_.end(), 0u);
    gen_ = 1;
  }
  out.clear();
  touched_.clear();
  run_sequence(t, bounds);
  // a pre-fill value that the fill overwrites is read from a saved copy
  auto snap_of = [&](int blk, int pos) {
    const size_t idx = static_cast<size_t>(blk) * nn_ + pos;
    if (snap_stamp_[idx] != gen_) {
      snap_stamp_[idx] = gen_;
      snap_row_[idx] = static_cast<int>(out.snaps.size());
      out.snaps.push_back(GhostSnap{slot[blk], pos});
    }
    return snap_row_[idx];
  };
  // a plain copy into an even position whose right neighbour is a plain copy
  // of the next source cell of the same block (not yet emitted) becomes one
  // paired op (same-level column and row copies, ~two thirds of a program)
  auto pairs_with = [&](int blk, int pos, const Desc &d) {
    if ((pos & 1) || (d.pos & 1)) return false;
    const size_t nxt = static_cast<size_t>(blk) * nn_ + pos + 1;
    if (stamp_[nxt] != gen_ || emit_stamp_[nxt] == gen_) return false;
    const Desc &e = cur_[nxt];
    if (e.type != GOP_COPY || e.blk != d.blk || e.pos != d.pos + 1) return false;
    if (e.blk == blk && e.pos == pos + 1) return false;  // unchanged cell
    return !overwritten(e.blk, e.pos);
  };
  out.ops.reserve(touched_.size());
  for (const int idx : touched_) {
    const Desc &d = cur_[idx];
    const int blk = idx / nn_, pos = idx % nn_;
    if (d.type == GOP_COPY && d.blk == blk && d.pos == pos) continue;  // unchanged
    if (emit_stamp_[idx] == gen_) continue;                             // second cell of a pair
    emit_stamp_[idx] = gen_;
    GhostOp op{};
    op.dst_slot = slot[blk];
    op.dst_pos = static_cast<int16_t>(pos);
    if (d.type == GOP_COPY) {
      if (overwritten(d.blk, d.pos)) {
        op.type = GOP_SNAP;
        op.src_slot = snap_of(d.blk, d.pos);
      } else {
        op.type = GOP_COPY;
        op.src_slot = slot[d.blk];
        op.src_pos = d.pos;
        if (pairs_with(blk, pos, d)) {
          op.type = GOP_COPY2;
          emit_stamp_[idx + 1] = gen_;
        }
      }
    } else {
      const int c[4] = {d.pos, d.pos + n_, d.pos + 1, d.pos + 1 + n_};  // sum_irjr order
      bool hazard = false;
      for (int q = 0; q < 4; q++) hazard |= overwritten(d.blk, c[q]);
      if (!hazard) {
        op.type = GOP_FINE;
        op.src_slot = slot[d.blk];
        op.src_pos = d.pos;
      } else {  // four consecutive rows, whether or not each was saved before
        op.type = GOP_SFINE;
        op.src_slot = static_cast<int>(out.snaps.size());
        for (int q = 0; q < 4; q++) out.snaps.push_back(GhostSnap{slot[d.blk], c[q]});
      }
    }
    out.ops.push_back(op);
  }
  group_by_block(t, slot, out);
}

// Stable counting sorts of the ops by destination block and of the
// snapshots by the block they save from (an SFINE's four rows stay
// consecutive), with the snapshot rows of the ops renumbered.
void GhostCompiler::group_by_block(const Tree &t, const int *slot, GhostProgram &out) {
  const int nb = t.lastActive;
  int top = 0;
  for (int b = 0; b < nb; b++) top = slot[b] > top ? slot[b] : top;
  if (static_cast<int>(blk_of_slot_.size()) <= top) blk_of_slot_.resize(static_cast<size_t>(top) + 1);
  for (int b = 0; b < nb; b++)
    if (slot[b] >= 0) blk_of_slot_[slot[b]] = b;
  bool leaves = true;
  auto sort = [&](auto &items, auto &tmp, std::vector<int> &start, auto slot_of, std::vector<int> *perm) {
    const size_t n = items.size();
    start.assign(static_cast<size_t>(nb) + 1, 0);
    for (size_t q = 0; q < n; q++) start[blk_of_slot_[slot_of(items[q])] + 1]++;
    for (int b = 0; b < nb; b++) {
      if (start[b + 1] && !t.leafs[b]) leaves = false;
      start[b + 1] += start[b];
    }
    count_.assign(start.begin(), start.end() - 1);
    tmp.resize(n);
    if (perm) perm->resize(n);
    for (size_t q = 0; q < n; q++) {
      const int g = count_[blk_of_slot_[slot_of(items[q])]]++;
      tmp[g] = items[q];
      if (perm) (*perm)[q] = g;
    }
    items.swap(tmp);
  };
  sort(out.snaps, snaps_tmp_, out.snap_start, [](const GhostSnap &s) { return s.slot; }, &snap_perm_);
  if (!out.snaps.empty())
    for (GhostOp &op : out.ops)
      if (op.type == GOP_SNAP || op.type == GOP_SFINE) op.src_slot = snap_perm_[op.src_slot];
  sort(out.ops, ops_tmp_, out.op_start, [](const GhostOp &o) { return o.dst_slot; }, nullptr);
  out.by_block = leaves;
}

}  // namespace amr
