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
