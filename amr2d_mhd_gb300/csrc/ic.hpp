// Initial conditions (IC2Dtype.cpp) evaluated on the host for the root blocks,
// plus the extension problems.  Not on the hot path: the result is uploaded
// once by amr_init.
#pragma once

#include <string>

namespace amr {

enum IcId { IC_SST = 0, IC_SST1, IC_SSTY, IC_BWX, IC_BWX1, IC_BWY, IC_BWY1, IC_ROTOR,
            IC_OT, IC_BLAST, IC_KH, IC_INVALID };

IcId ic_from_name(const std::string &name);

// gamma and tEnd chosen by the IC (IC2Dtype.cpp:20-78)
void ic_params(IcId ic, double &gamma, double &tend);

struct IcBlock {
  int n;          // block edge with ghosts
  int ng;
  int icoord_x, icoord_y;
  double dx, dy;  // of the block's level
  double shift_x, shift_y;  // subtracted from cell centres (dx[0] in the reference geometry)
};

// Primitive state W[8][n][n] (all cells, ghosts included) and face field
// Bi[2][n][n] from the cell averages (IC2Dtype.cpp:172-189).
void ic_fill(IcId ic, const double *ic_param, const IcBlock &b, double *W, double *Bi);

// W2U (meshblock.cpp:181-199) of one block, [8][n][n] arrays
void prim_to_cons(const double *W, double *U, int ncell, double gamma);

// max over interior cells of criteria.cpp:11-29 (relative jumps of p, rho,
// Bx, By) of one block given its primitive state
double criteria_grad(const double *W, int n, int ng);

}  // namespace amr

namespace amr {

// Seeded problem generators.  Draws come from MT19937-64 (the engine that
// std::mt19937_64 names, whose output sequence the C++ standard fixes) turned
// into doubles as (x >> 11) * 2^-53, so a seed gives the same problem on
// every platform.
class SeededDraw {
 public:
  explicit SeededDraw(unsigned long long seed);
  unsigned long long raw();
  double uniform();            // [0, 1)
  double normal();             // N(0, 1), Box-Muller (Box & Muller 1958)
 private:
  unsigned long long mt_[312];
  int idx_;
  bool have_spare_ = false;
  double spare_ = 0.0;
};

// Cylindrical blast instance `index` of the batch seeded by `seed`: generator
// seed = seed + index; draws in this order r0 ~ U[0.05, 0.15],
// p_in ~ U[5, 50], |B| ~ U[0.5, 2] / sqrt(4 pi), theta ~ U[0, pi/2],
// maxlevs ~ U{3..6}.  ic_param = {r0, p_in, |B|, theta, 0.5, 0.5}.
void blast_draw(unsigned long long seed, int index, double ic_param[6], int &maxlevs);

// Kelvin-Helmholtz perturbation amplitudes a_1..a_16 ~ N(0, sigma^2) with
// sigma = 1e-3, from the generator seeded with `seed`.
void kh_draw(unsigned long long seed, double a[16]);

}  // namespace amr
