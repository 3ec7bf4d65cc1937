/* Test infrastructure, not product code.
 *
 * The oracle: a plain-C, FP64, scalar restatement of the per-block
 * finite-volume update of spaceauk/AMR2D_MHD (reconstruction, Riemann fluxes,
 * residual + RK2, constrained transport, ghost fills, CFL dt, remeshing with
 * prolongation/restriction).  Every function cites the reference file:line it
 * follows.  It is used only by tests/, __graft_entry__.smoke() and the CPU
 * baseline leg of bench.py, as the checker of the CUDA path.
 *
 * Pinning: tests/golden/ holds state vectors produced by the reference itself
 * (built from its own sources by oracle/ref.mk); tests/test_oracle_golden.py
 * checks this restatement against them.
 *
 * Extensions beyond the reference (each off by default and marked where it
 * is used): N_x x N_y root blocks, periodic boundaries, a "clean" geometry
 * (dx = L / cells), gamma / tEnd overrides and the extra initial conditions
 * (MHD rotor with a free gamma, Orszag-Tang, seeded blast, seeded
 * Kelvin-Helmholtz).
 */
#ifndef AMR_ORACLE_H
#define AMR_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* reconstruction (input.txt `limiter`, slopelimiter.cpp:8-48, MUSCL2D.cpp:24-34) */
enum { OR_LIM_1ST = 0, OR_LIM_NOSL, OR_LIM_MINMOD, OR_LIM_VANLEER, OR_LIM_SUPERBEE,
       OR_LIM_MC, OR_LIM_KOREN, OR_LIM_CADA3RD, OR_LIM_WENO3, OR_LIM_WENO5 };
/* Riemann solver (input.txt `fluxMth`, riemannS.cpp:30-44) */
enum { OR_FLUX_RUSA = 0, OR_FLUX_HLLE, OR_FLUX_HLLC, OR_FLUX_HLLD, OR_FLUX_ROE };
/* initial conditions (IC2Dtype.cpp:18-168) + extensions */
enum { OR_IC_SST = 0, OR_IC_SST1, OR_IC_SSTY, OR_IC_BWX, OR_IC_BWX1, OR_IC_BWY,
       OR_IC_BWY1, OR_IC_ROTOR, OR_IC_ROTOR_B, OR_IC_OT, OR_IC_BLAST, OR_IC_KH };

typedef struct oracle_cfg {
  int nx_int, ny_int;    /* interior cells per block (input.txt line 1) */
  int nghosts;           /* defs.hpp:27 (2; 4 for WENO5) */
  int maxlevs;           /* defs.hpp:28 */
  int nroots_x, nroots_y;/* 2 x 2 in the reference (defs.hpp:29) */
  int periodic;          /* extension: 0 = mirror outflow (extboundary.cpp) */
  int geom_ref;          /* 1 = reference geometry (meshblock.cpp:90-91) */
  double lenx, leny, cfl;
  int ic, limiter, flux;
  double gamma_override; /* <= 0: the IC's own value */
  double tend_override;  /* <= 0: the IC's own value */
  double ic_param[24];   /* extension ICs: blast / KH parameters */
  int nthreads;          /* OpenMP threads over blocks (0 = default) */
  double dt_fixed;       /* extension: > 0 = every step uses this dt */
  int ct_type;           /* defs.hpp:34 CTtype: 1 (0 = 1) basic, 2 upwind EMF */
  int diffusion;         /* defs.hpp:35 diffusion: 0 off, 1 on */
} oracle_cfg;

/* what oracle_get copies */
enum { OR_GET_U = 0, OR_GET_US, OR_GET_W, OR_GET_FF, OR_GET_GG, OR_GET_BI, OR_GET_BIS,
       OR_GET_EMF, OR_GET_LP, OR_GET_ICOORD, OR_GET_LEAFS };

typedef struct oracle oracle;

oracle *oracle_create(const oracle_cfg *cfg);
void oracle_destroy(oracle *o);
int oracle_init(oracle *o);            /* basegrid + IC + W2U + initial admesh */
int oracle_step(oracle *o);            /* one iteration of main.cpp:128-247 */
int oracle_run(oracle *o, int nsteps, double t_stop);  /* steps until count==nsteps or t>t_stop */
int oracle_done(const oracle *o);      /* 1 when t > tEnd (loop exit of main.cpp:128) */
void oracle_info(const oracle *o, int *ints /*[8]*/, double *dbls /*[8]*/);
int64_t oracle_get(const oracle *o, int what, void *dst); /* returns #elements */
const char *oracle_error(const oracle *o);
/* overwrite the state arrays of blocks [0, lastActive) (what = U or BI) */
int oracle_set(oracle *o, int what, const double *src);

/* test hooks: skip the remesh at the end of oracle_step; run admesh alone */
void oracle_set_remesh(oracle *o, int on);
int oracle_admesh(oracle *o);
/* admesh with the caller's marks per block ID in place of criteria's */
int oracle_admesh_marked(oracle *o, const unsigned char *iref, const unsigned char *icoarse);

/* the sequential ghost fill of the current tree applied to `field` */
int oracle_fill(oracle *o, double *field, int nv, int kind);

/* unit-level entry points for known-answer tests */
double oracle_slopelimiter(int limiter, double r, double eta);
int oracle_riemann(int flux, const double *wL, const double *wR, double gamma, int dir_y,
                   double *out);
/* the same with the reference's compile-time MAG_field (defs.hpp:32) as an
 * argument: 0 is its hydrodynamic configuration, where ROE runs */
int oracle_riemann_mf(int flux, const double *wL, const double *wR, double gamma, int dir_y, int mag_field,
                      double *out);
void oracle_wavespeeds(const double *w, double gamma, int norm, double *out4);

#ifdef __cplusplus
}
#endif
#endif
