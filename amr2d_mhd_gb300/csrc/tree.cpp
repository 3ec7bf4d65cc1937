// Host quadtree: basegrid, locate_bounds and the tree logic of admesh.
#include "tree.hpp"

namespace amr {

namespace {
// side s: 0 left, 1 right, 2 bottom, 3 top; lp column of the neighbour
constexpr int kNbCol[4] = {4, 5, 6, 7};
constexpr int kOpp[4] = {1, 0, 3, 2};
constexpr int kBoxCode[4] = {-1, -2, -3, -4};
constexpr int kSameCode[4] = {1, 4, 7, 10};
constexpr int kFineCode[4] = {2, 5, 8, 11};
// first son of the finer neighbour that touches side s, and the step to the
// second one (locate_bounds.cpp:83-89, 123-124, 158-160, 194-195)
constexpr int kFineFirst[4] = {1, 0, 2, 0};
constexpr int kFineStep[4] = {2, 2, 1, 1};
}  // namespace

Tree::Tree(const TreeShape &s) : shape_(s) {
  // block IDs are never freed (admesh.cpp:33-51): a full tree bounds them
  long long per_root = 0, p = 1;
  for (int l = 0; l < s.maxlevs; l++) { per_root += p; p *= 4; }
  maxblocks_ = static_cast<int>(per_root * s.nrx * s.nry);
  lp.assign(maxblocks_, {0, 0, 0, 0, 0, 0, 0, 0});
  icoord.assign(maxblocks_, {0, 0});
  leafs.assign(maxblocks_, 0);
  iref.assign(maxblocks_, 0);
  icoarse.assign(maxblocks_, 0);
}

void Tree::basegrid() {
  const int nrx = shape_.nrx, nry = shape_.nry;
  const bool per = shape_.periodic;
  for (int jr = 0; jr < nry; jr++)
    for (int ir = 0; ir < nrx; ir++) {
      const int nb = jr * nrx + ir;
      auto &l = lp[nb];
      l[0] = 0; l[1] = 0; l[2] = 0; l[3] = 0;
      l[4] = ir > 0 ? nb - 1 : (per ? nb + nrx - 1 : -1);
      l[5] = ir < nrx - 1 ? nb + 1 : (per ? nb - (nrx - 1) : -1);
      l[6] = jr > 0 ? nb - nrx : (per ? nb + nrx * (nry - 1) : -1);
      l[7] = jr < nry - 1 ? nb + nrx : (per ? nb - nrx * (nry - 1) : -1);
      icoord[nb] = {ir * shape_.ni, jr * shape_.nj};
      leafs[nb] = 1;
      iref[nb] = 1;
    }
  lastActive = nrx * nry;
  nbleafs = lastActive;
  version++;
}

bool Tree::check(std::string &err) const {
  const int na = lastActive, nroots = shape_.nrx * shape_.nry;
  auto bad = [&](int b, const char *what) {
    err = "block " + std::to_string(b) + ": " + what;
    return false;
  };
  if (na < nroots || na > maxblocks_) {
    err = "last_active outside [nroots, maxblocks]";
    return false;
  }
  // index ranges (basegrid.cpp: roots are IDs 0..nroots-1 with father 0;
  // admesh.cpp:33-41: sons come as four consecutive IDs after the roots)
  for (int b = 0; b < na; b++) {
    const auto &l = lp[b];
    if (l[0] < 0 || l[0] >= shape_.maxlevs) return bad(b, "level outside [0, maxlevs)");
    if ((b < nroots) != (l[0] == 0)) return bad(b, "the roots are the first nrx * nry IDs, at level 0");
    if (l[1] < 0 || l[1] >= na) return bad(b, "father ID out of range");
    if (l[2] != 0 && (l[2] < nroots || l[2] + 3 >= na)) return bad(b, "first-son ID out of range");
    if (l[3] < 0 || l[3] > 3) return bad(b, "sibling number outside 0..3");
    for (int c = 4; c < 8; c++)
      if (l[c] < -1 || l[c] >= na) return bad(b, "neighbour ID out of range");
  }
  // father / son relations and the links inside each group of four sons
  // (updatelpup.cpp), which later remeshes follow
  for (int b = 0; b < na; b++) {
    const auto &l = lp[b];
    if (l[0] > 0) {
      const int f = l[1];
      if (lp[f][0] != l[0] - 1 || lp[f][2] + l[3] != b) return bad(b, "not the son its father lists");
      if (leafs[b] && leafs[f]) return bad(b, "a leaf whose father is a leaf");
    }
    if (l[2] != 0) {
      const int s = l[2];
      for (int q = 0; q < 4; q++)
        if (lp[s + q][0] != l[0] + 1 || lp[s + q][1] != b || lp[s + q][3] != q)
          return bad(b, "its sons do not list it as their father");
      if (lp[s][5] != s + 1 || lp[s][7] != s + 2 || lp[s + 1][4] != s || lp[s + 1][7] != s + 3 ||
          lp[s + 2][5] != s + 3 || lp[s + 2][6] != s || lp[s + 3][4] != s + 2 || lp[s + 3][6] != s + 1)
        return bad(b, "broken links between its sons");
    }
  }
  // the active tree (leaves and their ancestors): neighbours are active, on
  // the same level or, for a leaf, a leaf one level coarser; a leaf's
  // same-level neighbour that is refined has leaves along the shared edge
  std::vector<uint8_t> active(static_cast<size_t>(na), 0);
  for (int b = 0; b < na; b++)
    if (leafs[b])
      for (int a = b, depth = 0; depth < shape_.maxlevs && !active[a]; depth++) {
        active[a] = 1;
        if (lp[a][0] == 0) break;
        a = lp[a][1];
      }
  static constexpr int kFacing[4][2] = {{1, 3}, {0, 2}, {2, 3}, {0, 1}};  // sons of the L, R, D, U neighbour
  for (int b = 0; b < na; b++) {
    if (!active[b]) continue;
    if (!leafs[b] && lp[b][2] == 0) return bad(b, "a refined block without sons");
    for (int side = 0; side < 4; side++) {
      const int n = lp[b][kNbCol[side]];
      if (n == -1) continue;
      if (!active[n]) return bad(b, "a neighbour outside the active tree");
      if (lp[n][0] == lp[b][0] - 1 && leafs[b] && leafs[n]) continue;
      if (lp[n][0] != lp[b][0]) return bad(b, "a neighbour more than one level coarser, or finer");
      if (leafs[b] && !leafs[n])
        for (int k = 0; k < 2; k++)
          if (!leafs[lp[n][2] + kFacing[side][k]]) return bad(b, "neighbours two levels apart");
    }
  }
  return true;
}

std::vector<int> Tree::leaves() const {
  std::vector<int> out;
  for (int nb = 0; nb < lastActive; nb++)
    if (leafs[nb]) out.push_back(nb);
  return out;
}

void Tree::locate_bounds(std::vector<Bound> &out) const {
  out.clear();
  std::vector<std::array<uint8_t, 4>> done(lastActive, {0, 0, 0, 0});
  for (int nb = 0; nb < lastActive; nb++) {
    if (!leafs[nb]) continue;
    for (int s = 0; s < 4; s++) {
      if (done[nb][s]) continue;
      const int nbr = lp[nb][kNbCol[s]];
      if (nbr == -1) {
        done[nb][s] = 1;
        out.push_back({nb, -1, kBoxCode[s]});
      } else if (lp[nbr][0] >= lp[nb][0]) {
        if (leafs[nbr]) {
          out.push_back({nb, nbr, kSameCode[s]});
          done[nb][s] = 1;
          done[nbr][kOpp[s]] = 1;
        } else {
          done[nb][s] = 1;
          const int n1 = lp[nbr][2] + kFineFirst[s];
          const int n2 = n1 + kFineStep[s];
          out.push_back({nb, n1, kFineCode[s]});
          done[n1][kOpp[s]] = 1;
          done[n2][kOpp[s]] = 1;
        }
      }
      // a coarser neighbour fills this side from its own bound
    }
  }
}

// updatelpup.cpp:4-118.  Sons: 0 bottom-left, 1 bottom-right, 2 top-left,
// 3 top-right.  Outer sides of each son with the offset of the touching son
// of a refined neighbour.
void Tree::updatelpup(int nb, const int *s) {
  struct Outer { int q, side, off; };
  static constexpr Outer outer[8] = {{0, 0, 1}, {0, 2, 2}, {1, 1, 0}, {1, 2, 3},
                                     {2, 0, 3}, {2, 3, 0}, {3, 1, 2}, {3, 3, 1}};
  const int lev = lp[nb][0] + 1;
  for (int q = 0; q < 4; q++) {
    lp[s[q]][0] = lev;
    lp[s[q]][1] = nb;
    lp[s[q]][3] = q;
  }
  lp[s[0]][5] = s[1]; lp[s[0]][7] = s[2];
  lp[s[1]][4] = s[0]; lp[s[1]][7] = s[3];
  lp[s[2]][5] = s[3]; lp[s[2]][6] = s[0];
  lp[s[3]][4] = s[2]; lp[s[3]][6] = s[1];
  for (const Outer &o : outer) {
    const int col = kNbCol[o.side];
    const int nbr = lp[nb][col];
    if (nbr == -1 || leafs[nbr]) {
      lp[s[o.q]][col] = nbr;
    } else {
      const int nsr = lp[nbr][2] + o.off;
      lp[s[o.q]][col] = nsr;
      lp[nsr][kNbCol[kOpp[o.side]]] = s[o.q];
    }
  }
  leafs[nb] = 0;
  for (int q = 0; q < 4; q++) leafs[s[q]] = 1;
  nbleafs += 4;
  iref[nb] = 0;
  icoarse[nb] = 0;
  for (int q = 0; q < 4; q++) icoarse[s[q]] = 0;
}

// updatelpdown.cpp:4-54
void Tree::updatelpdown(int dad, const int *s) {
  leafs[dad] = 1;
  for (int q = 0; q < 4; q++) leafs[s[q]] = 0;
  nbleafs -= 3;
  int n = lp[dad][4];
  if (n != -1 && !leafs[n]) { n = lp[lp[n][2]][5]; lp[n][5] = dad; lp[lp[n][7]][5] = dad; }
  n = lp[dad][5];
  if (n != -1 && !leafs[n]) { n = lp[n][2]; lp[n][4] = dad; lp[lp[n][7]][4] = dad; }
  n = lp[dad][6];
  if (n != -1 && !leafs[n]) { n = lp[lp[n][2]][7]; lp[n][7] = dad; lp[lp[n][5]][7] = dad; }
  n = lp[dad][7];
  if (n != -1 && !leafs[n]) { n = lp[n][2]; lp[n][6] = dad; lp[lp[n][5]][6] = dad; }
}

bool Tree::admesh(const std::vector<double> &grad, AdmeshPlan &plan, std::string &err) {
  const int maxlevs = shape_.maxlevs;
  // markref.cpp:6-18 + criteria.cpp:31,43 (thresholds 0.05 / 1.0)
  for (int nb = 0; nb < lastActive; nb++) { iref[nb] = 0; icoarse[nb] = 0; }
  for (int nb = 0; nb < lastActive; nb++) {
    if (!leafs[nb] || lp[nb][0] < 0) continue;
    const double g = grad[nb];
    if (g >= 0.05) {
      if (lp[nb][0] < maxlevs - 1) { iref[nb] = 1; icoarse[nb] = 0; }
    } else if (g <= 1.0) {
      icoarse[nb] = 1;
    }
  }
  return apply_marks(plan, err);
}

bool Tree::admesh_marked(const uint8_t *mark_ref, const uint8_t *mark_crs, AdmeshPlan &plan, std::string &err) {
  const int maxlevs = shape_.maxlevs;
  // the marks as criteria.cpp:31-43 leaves them: leaves only, refinement
  // below the finest level, a refine mark cancelling a coarsen mark
  for (int nb = 0; nb < lastActive; nb++) { iref[nb] = 0; icoarse[nb] = 0; }
  for (int nb = 0; nb < lastActive; nb++) {
    if (!leafs[nb] || lp[nb][0] < 0) continue;
    if (mark_ref[nb]) {
      if (lp[nb][0] < maxlevs - 1) iref[nb] = 1;
    } else if (mark_crs[nb]) {
      icoarse[nb] = 1;
    }
  }
  return apply_marks(plan, err);
}

bool Tree::apply_marks(AdmeshPlan &plan, std::string &err) {
  const int maxlevs = shape_.maxlevs;
  plan.refine.clear();
  plan.coarsen.clear();
  // critneighup.cpp:6-34: keep neighbours within one level
  for (int nl = maxlevs - 1; nl >= 0; nl--)
    for (int nb = 0; nb < lastActive; nb++)
      if (iref[nb] && lp[nb][0] == nl)
        for (int c = 4; c < 8; c++) {
          const int n1 = lp[nb][c];
          if (n1 != -1 && lp[n1][0] < lp[nb][0]) iref[n1] = 1;
        }
  // refine, coarsest level first (admesh.cpp:30-59)
  for (int nl = 0; nl < maxlevs - 1; nl++)
    for (int nb = 0; nb < lastActive; nb++) {
      if (!(lp[nb][0] == nl && iref[nb])) continue;
      int s[4];
      if (lp[nb][2] == 0) {
        s[0] = lastActive; s[1] = s[0] + 1; s[2] = s[0] + 2; s[3] = s[0] + 3;
        lp[nb][2] = s[0];
        lastActive += 4;
        if (lastActive - 1 >= maxblocks_) {
          err = "nblocks exceeded max limit=" + std::to_string(maxblocks_);
          return false;
        }
      } else {
        s[0] = lp[nb][2]; s[1] = lp[s[0]][5]; s[2] = lp[s[0]][7]; s[3] = lp[s[2]][5];
      }
      // refine.cpp:61-84: son origins at the finer level
      const int x0 = icoord[nb][0] * 2, y0 = icoord[nb][1] * 2;
      icoord[s[0]] = {x0, y0};
      icoord[s[1]] = {x0 + shape_.ni, y0};
      icoord[s[2]] = {x0, y0 + shape_.nj};
      icoord[s[3]] = {x0 + shape_.ni, y0 + shape_.nj};
      plan.refine.push_back({nb, s[0], s[1], s[2], s[3]});
      updatelpup(nb, s);
    }
  // critneighdown.cpp:6-33
  for (int nb = 0; nb < lastActive; nb++)
    if (icoarse[nb])
      for (int c = 4; c < 8; c++) {
        const int n1 = lp[nb][c];
        if (n1 != -1 && !leafs[n1]) icoarse[nb] = 0;
      }
  // coarsen, finest level first (admesh.cpp:74-95)
  for (int nl = maxlevs - 1; nl >= 1; nl--)
    for (int nb = 0; nb < lastActive; nb++) {
      if (!(icoarse[nb] && lp[nb][3] == 0 && lp[nb][0] == nl)) continue;
      const int dad = lp[nb][1];
      int s[4] = {nb, lp[nb][5], lp[nb][7], 0};
      s[3] = lp[s[1]][7];
      if (icoarse[s[1]] && icoarse[s[2]] && icoarse[s[3]]) {
        plan.coarsen.push_back({dad, s[0], s[1], s[2], s[3]});
        updatelpdown(dad, s);
      }
    }
  if (!plan.refine.empty() || !plan.coarsen.empty()) version++;
  return true;
}

}  // namespace amr
