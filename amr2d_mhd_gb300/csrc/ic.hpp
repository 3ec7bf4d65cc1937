// Initial conditions (IC2Dtype.cpp) for the root blocks, plus the extension
// problems: the host prepares each block's constants and 1-D profiles, the
// device kernel k_ic (aux_kernels.cuh) fills the cells.
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

// One block of amr_init's initial condition as the device generator k_ic
// takes it.  The host fills what needs the C library's transcendental
// functions (IC2Dtype.cpp's sqrt(4 pi) constants, the blast field's cos /
// sin, the Orszag-Tang and Kelvin-Helmholtz profiles): every such function
// depends on x alone or on y alone, so the host evaluates it on the n cell
// centres of each direction (`tab`, three rows of n) and the device builds
// the n x n cells from those rows with the same arithmetic as before; the
// result is bit for bit the host evaluation's.
struct IcDev {
  int ic;                 // IcId
  int slot;               // physical slot of the block
  int icoord_x, icoord_y;
  double dx, dy, shift_x, shift_y;
  double gamma;
  double c[16];           // per IC: quadrant states r[4] p[4] bx[4] by[4] (SST*, BW*); rotor: c[0] =
                          // 2.5/sqrt(4 pi); OT: c[0] = rho, c[1] = p, c[2] = sqrt(4 pi); blast: r0, p_in,
                          // |B| cos(theta), |B| sin(theta), xc, yc; KH: c[0] = 0.1/sqrt(4 pi)
  int tab;                // first of this block's three table rows, -1 if none
  int pad;
};

// The IcDev and table rows [3][n] of one block: OT sin(x_i), sin(2 x_i),
// sin(y_j); KH the perturbation sum over k of a_k sin(2 pi k x_i), its
// envelope at y_j, unused.  Returns true if the block has table rows.
bool ic_prepare(IcId ic, const double *ic_param, const IcBlock &b, double gamma, IcDev &d, double *tab);

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
