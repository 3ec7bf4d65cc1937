/* Test infrastructure, not product code: the oracle (see amr_oracle.h).
 *
 * A scalar C11 restatement of spaceauk/AMR2D_MHD's time loop.  Citations are
 * file:line in that project.  Arrays are stored [block][var][j][i] (i fastest);
 * the reference stores Q[i][j][var][block] (meshblock.cpp:71-82), the values
 * and the order of every floating-point operation are the same.
 *
 * Compile with -ffp-contract=off: the reference's arithmetic is reproduced
 * operation by operation and must not be fused.
 */
#include "amr_oracle.h"

#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define EPS 1.0E-15             /* defs.hpp:16 */
#define PI_REF 3.14159265359    /* defs.hpp:23 */
#define MAXLEV 12

/* defs.hpp:110-111 macros and std::min/std::max: they differ for equal or
 * NaN arguments, so each call site uses the form the reference uses. */
static inline double MMIN(double a, double b) { return a < b ? a : b; }
static inline double MMAX(double a, double b) { return a > b ? a : b; }
static inline double SMIN(double a, double b) { return b < a ? b : a; }
static inline double SMAX(double a, double b) { return a < b ? b : a; }

enum { K_CC = 0, K_FC = 1, K_EC = 2 };

struct oracle {
  oracle_cfg c;
  int nx, ny, nv, ng;
  int nxmin, nxmax, nxminb, nxmaxb, nymin, nymax, nyminb, nymaxb, nxp1, nyp1, nx2, ny2;
  int nroots, maxblocks;
  double gamma, tEnd;
  double dx[MAXLEV], dy[MAXLEV];
  int (*lp)[8];
  int (*icoord)[2];
  unsigned char *leafs, *iref, *icoarse;
  int lastActive, nbleafs;
  int (*ib)[3];
  int nbounds, ib_cap;
  unsigned char *bflag;
  double *U, *Us, *W, *ff, *gg, *Bi, *Bis, *EMF;
  double t, dt, dtn;
  int count, done, initialised;
  int no_remesh;   /* test hook: skip the admesh at the end of a step */
  int nthreads;
  double *scratch;
  size_t cell, face;  /* doubles per block for a cell (8 vars) / face (2 comps) field */
  char err[512];
  int err_set;
};

typedef struct { double *a; int nv; int kind; } fld;

/* ---------------------------------------------------------------- errors */
static int fail(oracle *o, const char *msg) {
  int set = 0;
#ifdef _OPENMP
#pragma omp critical(oracle_err)
#endif
  {
    if (!o->err_set) { snprintf(o->err, sizeof(o->err), "%s", msg); o->err_set = 1; set = 1; }
  }
  (void)set;
  return -1;
}

/* -------------------------------------------------------------- indexing */
static inline size_t IX(const oracle *o, int nb, int nv, int k, int i, int j) {
  return ((((size_t)nb * nv) + k) * o->ny + j) * o->nx + i;
}
#define Qc(A, nb, k, i, j) (A)[IX(o, nb, 8, k, i, j)]
#define Qf(A, nb, k, i, j) (A)[IX(o, nb, 2, k, i, j)]
#define Qe(A, nb, i, j) (A)[IX(o, nb, 1, 0, i, j)]
#define F(f, nb, k, i, j) (f)->a[IX(o, nb, (f)->nv, k, i, j)]

/* ------------------------------------------------------ slopelimiter.cpp */
double oracle_slopelimiter(int limiter, double r, double eta) {
  /* slopelimiter.cpp:6-54 */
  double phi = 0.;
  switch (limiter) {
    case OR_LIM_1ST: phi = 0.; break;
    case OR_LIM_NOSL: phi = r; break;
    case OR_LIM_MINMOD: { double i0 = MMIN(1., r); phi = MMAX(0., i0); } break;
    case OR_LIM_VANLEER: phi = (fabs(r) + r) / (1. + fabs(r)); break;
    case OR_LIM_SUPERBEE: {
      double i0 = 2. * r;
      double i1 = MMIN(i0, 1.);
      i0 = MMIN(r, 2.);
      double i2 = MMAX(i0, i1);
      phi = MMAX(0., i2);
    } break;
    case OR_LIM_MC: {
      double i0 = 2. * r, i1 = 0.5 * (1. + r);
      double i2 = MMIN(i0, i1);
      i0 = MMIN(i2, 2.);
      phi = MMAX(0., i0);
    } break;
    case OR_LIM_KOREN: {
      double i0 = (1. + 2. * r) / 3.;
      double i1 = MMIN(i0, 2.);
      i0 = 2. * r;
      double i2 = MMIN(i0, i1);
      phi = MMAX(0., i2);
    } break;
    case OR_LIM_CADA3RD: {
      double i0 = MMIN(2. * r, (2. + r) / 3.);
      double i1 = MMIN(i0, 1.6);
      double ph = MMAX(-0.5 * r, i1);
      i0 = MMIN((2. + r) / 3., ph);
      ph = MMAX(0., i0);
      if (eta <= 1. - EPS) phi = (2. + r) / 3.;
      else if (eta >= 1. + EPS) phi = ph;
      else phi = 0.5 * ((1. - (eta - 1.) / EPS) * (2. + r) / 3. + (1 + (eta - 1.) / EPS) * ph);
    } break;
    default: phi = NAN; break;
  }
  return phi;
}

/* ------------------------------------------------------------- misc.cpp */
static inline double sgn(double v) { return v > 0 ? 1. : (v < 0 ? -1. : 0.); } /* misc.cpp:64-68 */

/* misc.cpp:71-79 */
static void wavespeeds(const double *w, double gamma, int norm, double *a, double *ca,
                       double *can, double *cf) {
  *ca = sqrt((w[5] * w[5] + w[6] * w[6] + w[7] * w[7]) / w[0]);
  *a = sqrt(gamma * w[4] / w[0]);
  *can = sqrt((w[norm] * w[norm]) / w[0]);
  double intm0 = (*ca * *ca) + (*a * *a);
  double intm1 = (*ca * *ca) - (*a * *a);
  *cf = sqrt(0.5 * (intm0 + sqrt(intm1 * intm1 + 4. * (*a * *a) * ((*ca * *ca) - (*can * *can)))));
}

void oracle_wavespeeds(const double *w, double gamma, int norm, double *out4) {
  wavespeeds(w, gamma, norm, &out4[0], &out4[1], &out4[2], &out4[3]);
}

/* misc.cpp:82-92 */
static void w2u(const double *w, double *u, double gamma) {
  u[0] = w[0];
  u[1] = w[0] * w[1];
  u[2] = w[0] * w[2];
  u[3] = w[0] * w[3];
  u[4] = w[4] / (gamma - 1) + 0.5 * w[0] * (w[1] * w[1] + w[2] * w[2] + w[3] * w[3]);
  u[4] += 0.5 * (w[5] * w[5] + w[6] * w[6] + w[7] * w[7]);
  u[5] = w[5]; u[6] = w[6]; u[7] = w[7];
}

/* misc.cpp:95-107 (note the sqrt(rhoL + sqrt(rhoR)) denominator, :98,100) */
static void roe_avg(const double *wL, const double *wR, double *RT, double *r, double *v,
                    double *B, double *Xfac, double *Yfac) {
  for (int i = 0; i < 3; i++) {
    v[i] = (sqrt(wL[0]) * wL[i + 1] + sqrt(wR[0]) * wR[i + 1]) / (sqrt(wL[0] + sqrt(wR[0])));
    B[i] = (sqrt(wL[0]) * wL[i + 5] + sqrt(wR[0]) * wR[i + 5]) / (sqrt(wL[0] + sqrt(wR[0])));
  }
  *RT = sqrt(wR[0] / wL[0]);
  *r = sqrt(wR[0] * wL[0]);
  double d6 = wL[6] - wR[6], d7 = wL[7] - wR[7];
  *Xfac = 0.5 * (d6 * d6 + d7 * d7) / (sqrt(wL[0]) + sqrt(wR[0]));
  *Yfac = 0.5 * (wL[0] + wR[0]) / *r;
}

/* misc.cpp:110-140; only lambda[0] and lambda[6] are used by the callers */
static void roe_eigen(double gamma, double d, const double *v, double h, const double *B,
                      double Xfac, double Yfac, double *lam) {
  double vsq = v[0] * v[0] + v[1] * v[1] + v[2] * v[2];
  double btsq = B[1] * B[1] + B[2] * B[2];
  double bt_starsq = (gamma - 1. - (gamma - 2) * Yfac) * btsq;
  double vaxsq = B[0] * B[0] / d;
  double vax = sqrt(vaxsq);
  double hp = h - (vaxsq + btsq / d);
  double twid_asq = ((gamma - 1.) * (hp - 0.5 * vsq) - (gamma - 2.) * Xfac);
  twid_asq = MMAX(twid_asq, EPS);
  double ct2 = bt_starsq / d;
  double tsum = vaxsq + ct2 + twid_asq;
  double tdif = vaxsq + ct2 - twid_asq;
  double cf2_cs2 = sqrt(tdif * tdif + 4. * twid_asq * ct2);
  double cfsq = 0.5 * (tsum + cf2_cs2);
  double cfast = sqrt(cfsq);
  double cssq = twid_asq * vaxsq / cfsq;
  double cslow = sqrt(cssq);
  lam[0] = v[0] - cfast;
  lam[1] = v[0] - vax;
  lam[2] = v[0] - cslow;
  lam[3] = v[0];
  lam[4] = v[0] + cslow;
  lam[5] = v[0] + vax;
  lam[6] = v[0] + cfast;
}

/* ---------------------------------------------------------- riemannS.cpp */
/* The common preamble of RUSA/HLLE/HLLC/HLLD (riemannS.cpp:59-108 and
 * repeats): conserved states q, physical fluxes F, enthalpy, total pressure. */
typedef struct { double q[8], F[8], H, pt, cf, e; } side_t;

static void side_state(const double *w, double gamma, side_t *s) {
  double a, ca, can;
  wavespeeds(w, gamma, 5, &a, &ca, &can, &s->cf);
  double vn = w[1], Bn = w[5];
  double e = (w[4] / (w[0] * (gamma - 1))) + 0.5 * (w[1] * w[1] + w[2] * w[2] + w[3] * w[3]) +
             0.5 * (w[5] * w[5] + w[6] * w[6] + w[7] * w[7]) / w[0];
  e = e * w[0];
  s->e = e;
  s->H = (e + w[4] + 0.5 * (w[5] * w[5] + w[6] * w[6] + w[7] * w[7])) / w[0];
  for (int k = 0; k < 8; k++) s->q[k] = w[k];
  s->q[1] = w[0] * w[1]; s->q[2] = w[0] * w[2]; s->q[3] = w[0] * w[3];
  s->q[4] = e;
  double pt = w[4] + 0.5 * (w[5] * w[5] + w[6] * w[6] + w[7] * w[7]);
  s->pt = pt;
  s->F[0] = w[0] * vn;
  s->F[1] = w[0] * vn * w[1] + pt - Bn * w[5];
  s->F[2] = w[0] * vn * w[2] - Bn * w[6];
  s->F[3] = w[0] * vn * w[3] - Bn * w[7];
  s->F[4] = w[0] * vn * s->H - Bn * (w[1] * w[5] + w[2] * w[6] + w[3] * w[7]);
  s->F[5] = vn * w[5] - Bn * w[1];
  s->F[6] = vn * w[6] - Bn * w[2];
  s->F[7] = vn * w[7] - Bn * w[3];
}

/* riemannS.cpp:58-116 */
static int rusa(const double *wL, const double *wR, double gamma, double *flux) {
  side_t L, R;
  side_state(wL, gamma, &L);
  side_state(wR, gamma, &R);
  double i2 = L.cf + fabs(wL[1]), i3 = R.cf + fabs(wR[1]);
  double im = SMAX(i2, i3);
  for (int k = 0; k < 8; k++) flux[k] = 0.5 * (L.F[k] + R.F[k]) - 0.5 * im * (R.q[k] - L.q[k]);
  return 0;
}

/* riemannS.cpp:118-189 */
static int hlle(const double *wL, const double *wR, double gamma, double *flux) {
  side_t L, R;
  side_state(wL, gamma, &L);
  side_state(wR, gamma, &R);
  double v[3], B[3], RT, r, Xf, Yf, lam[7];
  roe_avg(wL, wR, &RT, &r, v, B, &Xf, &Yf);
  double H = (L.H + RT * R.H) / (1 + RT);
  roe_eigen(gamma, r, v, H, B, Xf, Yf, lam);
  double SL = SMIN(wL[1] - L.cf, lam[0]);
  SL = MMIN(SL, 0.);
  double SR = SMAX(wR[1] + R.cf, lam[6]);
  SR = MMAX(SR, 0.);
  for (int k = 0; k < 8; k++)
    flux[k] = (SR * L.F[k] - SL * R.F[k] + SL * SR * (R.q[k] - L.q[k])) / (SR - SL);
  return 0;
}

/* riemannS.cpp:192-295 (Linde 1998) */
static int hllc(const double *wL, const double *wR, double gamma, double *flux) {
  side_t L, R;
  side_state(wL, gamma, &L);
  side_state(wR, gamma, &R);
  double v[3], B[3], RT, r, Xf, Yf, lam[7];
  roe_avg(wL, wR, &RT, &r, v, B, &Xf, &Yf);
  double H = (L.H + RT * R.H) / (1 + RT);
  roe_eigen(gamma, r, v, H, B, Xf, Yf, lam);
  double SL = SMIN(wL[1] - L.cf, lam[0]);
  double SR = SMAX(wR[1] + R.cf, lam[6]);
  double SM = v[0];
  double s1 = 0., s2 = 0.;
  for (int k = 0; k < 8; k++) s1 += fabs(R.q[k] - L.q[k]);
  for (int k = 0; k < 8; k++) s2 += fabs((R.F[k] - L.F[k]) - v[0] * (R.q[k] - L.q[k]));
  double interm = 1. - s2 / (s1 + EPS);
  double alpha = MMAX(0., interm);
  if (alpha > 1 || alpha < 0 || isnan(alpha)) return -2;   /* riemannS.cpp:269-272 */
  if (SR - SL == 0) return -3;                              /* riemannS.cpp:273-276 */
  double FLs[8], FRs[8];
  for (int k = 0; k < 8; k++) {
    FLs[k] = ((SL * ((1 - alpha) * SR + alpha * v[0])) / (SR - SL)) * (R.q[k] - L.q[k]) -
             (SL / (SR - SL)) * R.F[k] + ((SR) / (SR - SL)) * L.F[k];
    FRs[k] = ((SR * ((1 - alpha) * SL + alpha * v[0])) / (SR - SL)) * (R.q[k] - L.q[k]) -
             (SL / (SR - SL)) * R.F[k] + ((SR) / (SR - SL)) * L.F[k];
  }
  for (int k = 0; k < 8; k++) {
    if (SL > 0.) flux[k] = L.F[k];
    else if (SL <= 0. && SM >= 0.) flux[k] = FLs[k];
    else if (SM <= 0. && SR >= 0.) flux[k] = FRs[k];
    else if (SR < 0.) flux[k] = R.F[k];
  }
  return 0;
}

static inline double dot13_57(const double *a) { /* misc.cpp:51-61, dot_prod(v,1,3,v,5,7) */
  double s = 0.;
  s += a[1] * a[5];
  s += a[2] * a[6];
  s += a[3] * a[7];
  return s;
}

/* riemannS.cpp:397-549 (Miyoshi & Kusano 2005) */
static int hlld(const double *wL, const double *wR, double gamma, double *flux) {
  side_t L, R;
  side_state(wL, gamma, &L);
  side_state(wR, gamma, &R);
  double wLs[8] = {0}, wLss[8] = {0}, wRs[8] = {0}, wRss[8] = {0};
  double qLs[8], qLss[8], qRs[8], qRss[8];
  double vnL = wL[1], vnR = wR[1], ptL = L.pt, ptR = R.pt;
  double SL = SMIN(vnL, vnR) - SMAX(L.cf, R.cf);
  double SR = SMAX(vnL, vnR) + SMAX(L.cf, R.cf);
  double SM = ((SR - vnR) * wR[0] * vnR - (SL - vnL) * wL[0] * vnL - ptR + ptL) /
              ((SR - vnR) * wR[0] - (SL - vnL) * wL[0]);
  double pts = ((SR - vnR) * wR[0] * ptL - (SL - vnL) * wL[0] * ptR +
                wL[0] * wR[0] * (SR - vnR) * (SL - vnL) * (vnR - vnL)) /
               ((SR - vnR) * wR[0] - (SL - vnL) * wL[0]);
  /* left * (:467-481) */
  wLs[0] = wL[0] * (SL - vnL) / (SL - SM);
  wLs[1] = SM;
  wLs[5] = wL[5];
  if ((wL[0] * (SL - wL[1]) * (SL - SM) - wL[5] * wL[5]) != 0) {
    double den = wL[0] * (SL - wL[1]) * (SL - SM) - wL[5] * wL[5];
    wLs[2] = wL[2] - wL[5] * wL[6] * ((SM - wL[1]) / den);
    wLs[3] = wL[3] - wL[5] * wL[7] * ((SM - wL[1]) / den);
    wLs[6] = wL[6] * ((wL[0] * ((SL - wL[1]) * (SL - wL[1])) - wL[5] * wL[5]) / den);
    wLs[7] = wL[7] * ((wL[0] * ((SL - wL[1]) * (SL - wL[1])) - wL[5] * wL[5]) / den);
  } else {
    wLs[2] = wL[2]; wLs[3] = wL[3]; wLs[6] = 0.; wLs[7] = 0.;
  }
  double eLs = (((SL - wL[1]) * L.e - ptL * wL[1] + pts * SM + wL[5] * (dot13_57(wL) - dot13_57(wLs))) /
                (SL - SM));
  /* right * (:483-497) */
  wRs[0] = wR[0] * (SR - vnR) / (SR - SM);
  wRs[1] = SM;
  wRs[5] = wR[5];
  if ((wR[0] * (SR - wR[1]) * (SR - SM) - wR[5] * wR[5]) != 0) {
    double den = wR[0] * (SR - wR[1]) * (SR - SM) - wR[5] * wR[5];
    wRs[2] = wR[2] - wR[5] * wR[6] * ((SM - wR[1]) / den);
    wRs[3] = wR[3] - wR[5] * wR[7] * ((SM - wR[1]) / den);
    wRs[6] = wR[6] * ((wR[0] * ((SR - wR[1]) * (SR - wR[1])) - wR[5] * wR[5]) / den);
    wRs[7] = wR[7] * ((wR[0] * ((SR - wR[1]) * (SR - wR[1])) - wR[5] * wR[5]) / den);
  } else {
    wRs[2] = wR[2]; wRs[3] = wR[3]; wRs[6] = 0; wRs[7] = 0;
  }
  double eRs = (((SR - wR[1]) * R.e - ptR * wR[1] + pts * SM + wR[5] * (dot13_57(wR) - dot13_57(wRs))) /
                (SR - SM));
  /* ** states (:501-519) */
  double sLs = sqrt(wLs[0]), sRs = sqrt(wRs[0]);
  wLss[0] = wLs[0];
  wLss[1] = SM;
  wLss[2] = (sLs * wLs[2] + sRs * wRs[2] + (wRs[6] - wLs[6]) * sgn(wL[5])) / (sLs + sRs);
  wLss[3] = (sLs * wLs[3] + sRs * wRs[3] + (wRs[7] - wLs[7]) * sgn(wL[5])) / (sLs + sRs);
  wLss[5] = wLs[5];
  wLss[6] = (sLs * wRs[6] + sRs * wLs[6] + sqrt(wLs[0] * wRs[0]) * (wRs[2] - wLs[2]) * sgn(wL[5])) /
            (sLs + sRs);
  wLss[7] = (sLs * wRs[7] + sRs * wLs[7] + sqrt(wLs[0] * wRs[0]) * (wRs[3] - wLs[3]) * sgn(wL[5])) /
            (sLs + sRs);
  double eLss = eLs - sLs * (dot13_57(wLs) - dot13_57(wLss)) * sgn(wL[5]);
  for (int k = 0; k < 8; k++) wRss[k] = wLss[k];
  double eRss = eRs + sRs * (dot13_57(wRs) - dot13_57(wRss)) * sgn(wR[5]);
  w2u(wLs, qLs, gamma);
  w2u(wLss, qLss, gamma);
  qLs[4] = eLs; qLss[4] = eLss;
  w2u(wRs, qRs, gamma);
  w2u(wRss, qRss, gamma);
  qRs[4] = eRs; qRss[4] = eRss;
  double SLs = SM - fabs(wL[5]) / sLs;
  double SRs = SM + fabs(wR[5]) / sRs;
  for (int k = 0; k < 8; k++) {
    if (SL > 0) flux[k] = L.F[k];
    else if (SL <= 0. && SLs >= 0.) flux[k] = L.F[k] + SL * qLs[k] - SL * L.q[k];
    else if (SLs <= 0. && SM >= 0.) flux[k] = L.F[k] + SLs * qLss[k] - (SLs - SL) * qLs[k] - SL * L.q[k];
    else if (SM <= 0. && SRs >= 0.) flux[k] = R.F[k] + SRs * qRss[k] - (SRs - SR) * qRs[k] - SR * R.q[k];
    else if (SRs <= 0. && SR >= 0.) flux[k] = R.F[k] + SR * qRs[k] - SR * R.q[k];
    else if (SR < 0.) flux[k] = R.F[k];
  }
  return 0;
}

/* riemannS.cpp:297-395, the hydrodynamic Roe solver (Toro, p. 376); the
 * normal is x (xnorm = 1, ynorm = 0, written out as the reference does) and
 * the field enters the physical fluxes only.  (gamma-1)/pow(a,2) as the
 * reference writes it (:366). */
static int roe(const double *wL, const double *wR, double gamma, double *flux) {
  const double xnorm = 1.0, ynorm = 0.0;
  double vnL = wL[1] * xnorm + wL[2] * ynorm, BnL = wL[5] * xnorm + wL[6] * ynorm;
  double eL = (wL[4] / (wL[0] * (gamma - 1))) + 0.5 * (wL[1] * wL[1] + wL[2] * wL[2] + wL[3] * wL[3]) +
              0.5 * (wL[5] * wL[5] + wL[6] * wL[6] + wL[7] * wL[7]) / wL[0];
  eL = eL * wL[0];
  double HL = (eL + wL[4] + 0.5 * (wL[5] * wL[5] + wL[6] * wL[6] + wL[7] * wL[7])) / wL[0];
  double qL[8], qR[8], FL[8], FR[8];
  for (int k = 0; k < 8; k++) { qL[k] = wL[k]; qR[k] = wR[k]; }
  qL[1] = wL[0] * wL[1]; qL[2] = wL[0] * wL[2]; qL[3] = wL[0] * wL[3]; qL[4] = eL;
  double vnR = wR[1] * xnorm + wR[2] * ynorm, BnR = wR[5] * xnorm + wR[6] * ynorm;
  double eR = (wR[4] / (wR[0] * (gamma - 1))) + 0.5 * (wR[1] * wR[1] + wR[2] * wR[2] + wR[3] * wR[3]) +
              0.5 * (wR[5] * wR[5] + wR[6] * wR[6] + wR[7] * wR[7]) / wR[0];
  eR = eR * wR[0];
  double HR = (eR + wR[4] + 0.5 * (wR[5] * wR[5] + wR[6] * wR[6] + wR[7] * wR[7])) / wR[0];
  qR[1] = wR[0] * wR[1]; qR[2] = wR[0] * wR[2]; qR[3] = wR[0] * wR[3]; qR[4] = eR;
  /* 1) Roe averages */
  double RT = sqrt(wR[0] / wL[0]);
  double u = (wL[1] + RT * wR[1]) / (1 + RT);
  double v = (wL[2] + RT * wR[2]) / (1 + RT);
  double w = (wL[3] + RT * wR[3]) / (1 + RT);
  double H = (HL + RT * HR) / (1 + RT);
  double a = sqrt((gamma - 1) * (H - 0.5 * (u * u + v * v + w * w)));
  /* 2) eigenvalues, 3) right eigenvectors */
  double lambda[5] = {u - a, u, u, u, u + a};
  double K[5][8] = {{1., u - a, v, w, H - u * a, 0., 0., 0.},
                    {1., u, v, w, 0.5 * (u * u + v * v + w * w), 0., 0., 0.},
                    {0., 0., 1., 0., v, 0., 0., 0.},
                    {0., 0., 0., 1., w, 0., 0., 0.},
                    {1., u + a, v, w, H + u * a, 0., 0., 0.}};
  /* 4) wave strengths */
  double alpha[5];
  alpha[2] = (qR[2] - qL[2]) - v * (qR[0] - qL[0]);
  alpha[3] = (qR[3] - qL[3]) - w * (qR[0] - qL[0]);
  double du5bar = (qR[4] - qL[4]) - (alpha[2]) * v - (alpha[3]) * w;
  alpha[1] = ((gamma - 1) / pow(a, 2)) * ((qR[0] - qL[0]) * (H - u * u) + u * (qR[1] - qL[1]) - du5bar);
  alpha[0] = 0.5 * (1 / a) * ((qR[0] - qL[0]) * (u + a) - (qR[1] - qL[1]) - a * alpha[1]);
  alpha[4] = (qR[0] - qL[0]) - (alpha[0] + alpha[1]);
  /* 5) physical fluxes and the Roe flux */
  double ptL = wL[4] + 0.5 * (wL[5] * wL[5] + wL[6] * wL[6] + wL[7] * wL[7]);
  FL[0] = wL[0] * vnL;
  FL[1] = wL[0] * vnL * wL[1] + xnorm * ptL - BnL * wL[5];
  FL[2] = wL[0] * vnL * wL[2] + ynorm * ptL - BnL * wL[6];
  FL[3] = wL[0] * vnL * wL[3] - BnL * wL[7];
  FL[4] = wL[0] * vnL * HL - BnL * (wL[1] * wL[5] + wL[2] * wL[6] + wL[3] * wL[7]);
  FL[5] = vnL * wL[5] - BnL * wL[1];
  FL[6] = vnL * wL[6] - BnL * wL[2];
  FL[7] = vnL * wL[7] - BnL * wL[3];
  double ptR = wR[4] + 0.5 * (wR[5] * wR[5] + wR[6] * wR[6] + wR[7] * wR[7]);
  FR[0] = wR[0] * vnR;
  FR[1] = wR[0] * vnR * wR[1] + xnorm * ptR - BnR * wR[5];
  FR[2] = wR[0] * vnR * wR[2] + ynorm * ptR - BnR * wR[6];
  FR[3] = wR[0] * vnR * wR[3] - BnR * wR[7];
  FR[4] = wR[0] * vnR * HR - BnR * (wR[1] * wR[5] + wR[2] * wR[6] + wR[3] * wR[7]);
  FR[5] = vnR * wR[5] - BnR * wR[1];
  FR[6] = vnR * wR[6] - BnR * wR[2];
  FR[7] = vnR * wR[7] - BnR * wR[3];
  for (int k = 0; k < 8; k++) {
    double summ = 0.;
    for (int j = 0; j < 5; j++) summ += alpha[j] * fabs(lambda[j]) * K[j][k];
    flux[k] = 0.5 * (FL[k] + FR[k]) - 0.5 * summ;
  }
  return 0;
}

/* riemannS.cpp:7-56: rotate y faces (the field components only with
 * MAG_field, :18,51), dispatch, rotate back.  ROE is rejected with a
 * magnetic field (riemannS.cpp:39-40); the time loop always runs with
 * MAG_field (defs.hpp:32), the hydrodynamic configuration is reachable here
 * through mag_field = 0. */
int oracle_riemann_mf(int fluxm, const double *wL, const double *wR, double gamma, int dir_y, int mag_field,
                      double *out) {
  double l[8], r[8], f[8] = {0};
  for (int k = 0; k < 8; k++) { l[k] = wL[k]; r[k] = wR[k]; }
  if (dir_y) {
    l[1] = wL[2]; l[2] = wL[1]; r[1] = wR[2]; r[2] = wR[1];
    if (mag_field) { l[5] = wL[6]; l[6] = wL[5]; r[5] = wR[6]; r[6] = wR[5]; }
  }
  int rc;
  switch (fluxm) {
    case OR_FLUX_RUSA: rc = rusa(l, r, gamma, f); break;
    case OR_FLUX_HLLE: rc = hlle(l, r, gamma, f); break;
    case OR_FLUX_HLLC: rc = hllc(l, r, gamma, f); break;
    case OR_FLUX_HLLD: rc = hlld(l, r, gamma, f); break;
    case OR_FLUX_ROE:
      if (mag_field) return -4;
      rc = roe(l, r, gamma, f);
      break;
    default: return -4;
  }
  if (rc) return rc;
  for (int k = 0; k < 8; k++) out[k] = f[k];
  if (dir_y) {
    out[1] = f[2]; out[2] = f[1];
    if (mag_field) { out[5] = f[6]; out[6] = f[5]; }
  }
  return 0;
}

int oracle_riemann(int fluxm, const double *wL, const double *wR, double gamma, int dir_y, double *out) {
  return oracle_riemann_mf(fluxm, wL, wR, gamma, dir_y, 1, out);
}

/* ---------------------------------------------------------- meshblock.cpp */
/* meshblock.cpp:119-179: U2W (check_nan=0) and Us2W (check_nan=1) over the
 * whole block, with the pressure trap on i,j in (nxminb, nxmaxb). */
static int cons2prim(oracle *o, const double *Q, int nb, int check_nan) {
  double g = o->gamma;
  for (int i = 0; i < o->nx; i++)
    for (int j = 0; j < o->ny; j++) {
      double u0 = Qc(Q, nb, 0, i, j);
      double w0 = u0, w1 = Qc(Q, nb, 1, i, j) / u0, w2 = Qc(Q, nb, 2, i, j) / u0,
             w3 = Qc(Q, nb, 3, i, j) / u0;
      double w4 = (g - 1) * (Qc(Q, nb, 4, i, j) - 0.5 * w0 * (w1 * w1 + w2 * w2 + w3 * w3));
      double b5 = Qc(Q, nb, 5, i, j), b6 = Qc(Q, nb, 6, i, j), b7 = Qc(Q, nb, 7, i, j);
      w4 = w4 - (g - 1) * (0.5 * (b5 * b5 + b6 * b6 + b7 * b7));
      Qc(o->W, nb, 0, i, j) = w0; Qc(o->W, nb, 1, i, j) = w1; Qc(o->W, nb, 2, i, j) = w2;
      Qc(o->W, nb, 3, i, j) = w3; Qc(o->W, nb, 4, i, j) = w4; Qc(o->W, nb, 5, i, j) = b5;
      Qc(o->W, nb, 6, i, j) = b6; Qc(o->W, nb, 7, i, j) = b7;
      if (w4 <= 0 && i > o->nxminb && i < o->nxmaxb && j > o->nyminb && j < o->nymaxb) {
        char m[160];
        snprintf(m, sizeof m, "non-positive pressure %g at block %d cell (%d,%d)", w4, nb, i, j);
        return fail(o, m);
      }
      if (check_nan && (isnan(w1) || isnan(w2) || isnan(w3)))
        return fail(o, "NaN velocity in Us2W");
    }
  return 0;
}

/* meshblock.cpp:181-199 */
static void prim2cons(oracle *o, int nb) {
  double g = o->gamma;
  for (int i = 0; i < o->nx; i++)
    for (int j = 0; j < o->ny; j++) {
      double w[8];
      for (int k = 0; k < 8; k++) w[k] = Qc(o->W, nb, k, i, j);
      Qc(o->U, nb, 0, i, j) = w[0];
      Qc(o->U, nb, 1, i, j) = w[1] * w[0];
      Qc(o->U, nb, 2, i, j) = w[2] * w[0];
      Qc(o->U, nb, 3, i, j) = w[3] * w[0];
      double e = (w[4] / (g - 1)) + 0.5 * w[0] * (w[1] * w[1] + w[2] * w[2] + w[3] * w[3]);
      Qc(o->U, nb, 5, i, j) = w[5];
      Qc(o->U, nb, 6, i, j) = w[6];
      Qc(o->U, nb, 7, i, j) = w[7];
      Qc(o->U, nb, 4, i, j) = e + 0.5 * (w[5] * w[5] + w[6] * w[6] + w[7] * w[7]);
    }
}

/* ------------------------------------------------- celledges.cpp / WENO */
typedef struct { double *dwdx, *dwdy, *wxL, *wxR, *wyL, *wyR; } scr_t;
#define S(a, k, i, j) (a)[(((size_t)(k)) * o->ny + (j)) * o->nx + (i)]

static scr_t thread_scratch(oracle *o) {
  int tid = 0;
#ifdef _OPENMP
  tid = omp_get_thread_num();
#endif
  size_t n = (size_t)8 * o->nx * o->ny;
  double *b = o->scratch + (size_t)tid * 6 * n;
  scr_t s = {b, b + n, b + 2 * n, b + 3 * n, b + 4 * n, b + 5 * n};
  return s;
}

/* celledges.cpp:5-66 */
static int celledges(oracle *o, int nb, scr_t *s) {
  int nx = o->nx, ny = o->ny, lim = o->c.limiter;
  const double *W = o->W;
  for (int i = 0; i < nx; i++)
    for (int j = 0; j < ny; j++)
      for (int k = 0; k < 8; k++) {
        int im = i > 0 ? i - 1 : i, jm = j > 0 ? j - 1 : j;
        int ii = im + 1, jj = jm + 1;
        S(s->dwdx, k, i, j) = Qc(W, nb, k, ii, j) - Qc(W, nb, k, im, j);
        S(s->dwdy, k, i, j) = Qc(W, nb, k, i, jj) - Qc(W, nb, k, i, jm);
        if (isnan(S(s->dwdx, k, i, j)) || isnan(S(s->dwdy, k, i, j)))
          return fail(o, "NaN in celledges differences");
      }
  double lv = (double)o->dx[o->lp[nb][0]], lvy = o->dy[o->lp[nb][0]];
  for (int i = 0; i < nx - 1; i++)
    for (int j = 0; j < ny - 1; j++)
      for (int k = 0; k < 8; k++) {
        double r, phi, eta;
        if (k != 5) {
          if (lim == OR_LIM_CADA3RD) {
            double a = S(s->dwdx, k, i + 1, j), b = S(s->dwdx, k, i, j);
            eta = (a * a + b * b) / ((1 * lv) * (1 * lv));
          } else eta = 0.;
          r = S(s->dwdx, k, i + 1, j) / (S(s->dwdx, k, i, j) + EPS);
          phi = oracle_slopelimiter(lim, r, eta);
          S(s->wxL, k, i, j) = Qc(W, nb, k, i, j) + 0.5 * phi * S(s->dwdx, k, i, j);
          r = S(s->dwdx, k, i, j) / (S(s->dwdx, k, i + 1, j) + EPS);
          phi = oracle_slopelimiter(lim, r, eta);
          S(s->wxR, k, i, j) = Qc(W, nb, k, i, j) - 0.5 * phi * S(s->dwdx, k, i + 1, j);
          if (isnan(S(s->wxL, k, i, j))) return fail(o, "NaN in celledges face state");
        }
        if (k != 6) {
          if (lim == OR_LIM_CADA3RD) {
            double a = S(s->dwdy, k, i, j + 1), b = S(s->dwdy, k, i, j);
            eta = (a * a + b * b) / ((1 * lvy) * (1 * lvy));
          } else eta = 0.;
          r = S(s->dwdy, k, i, j + 1) / (S(s->dwdy, k, i, j) + EPS);
          phi = oracle_slopelimiter(lim, r, eta);
          S(s->wyL, k, i, j) = Qc(W, nb, k, i, j) + 0.5 * phi * S(s->dwdy, k, i, j);
          r = S(s->dwdy, k, i, j) / (S(s->dwdy, k, i, j + 1) + EPS);
          phi = oracle_slopelimiter(lim, r, eta);
          S(s->wyR, k, i, j) = Qc(W, nb, k, i, j) - 0.5 * phi * S(s->dwdy, k, i, j + 1);
        }
      }
  return 0;
}

/* WENO2D_primvar.cpp:7-91 */
static void weno3(oracle *o, int nb, int diry, scr_t *s) {
  const double e = 1.E-15;
  for (int i = o->nxminb; i <= o->nxmaxb; i++)
    for (int j = o->nyminb; j <= o->nymaxb; j++)
      for (int k = 0; k < 8; k++) {
        if (!diry && k == 5) continue;
        if (diry && k == 6) continue;
        int ip = diry ? i : i + 1, jp = diry ? j + 1 : j;
        int im = diry ? i : i - 1, jm = diry ? j - 1 : j;
        double w = Qc(o->W, nb, k, i, j), wp = Qc(o->W, nb, k, ip, jp), wm = Qc(o->W, nb, k, im, jm);
        double p0n = 0.5 * wm + 0.5 * w, p1n = 1.5 * w - 0.5 * wp;
        double B0n = (w - wm) * (w - wm), B1n = (wp - w) * (wp - w);
        double d0n = 2. / 3., d1n = 1. / 3.;
        double a0n = d0n / ((e + B0n) * (e + B0n)), a1n = d1n / ((e + B1n) * (e + B1n));
        double asn = a0n + a1n;
        double w0n = a0n / asn, w1n = a1n / asn;
        double vR = w0n * p0n + w1n * p1n;
        double p0p = 1.5 * w - 0.5 * wm, p1p = 0.5 * wp + 0.5 * w;
        double B0p = (w - wm) * (w - wm), B1p = (wp - w) * (wp - w);
        double d0p = 1. / 3., d1p = 2. / 3.;
        double a0p = d0p / ((e + B0p) * (e + B0p)), a1p = d1p / ((e + B1p) * (e + B1p));
        double asp = a0p + a1p;
        double w0p = a0p / asp, w1p = a1p / asp;
        double vL = w0p * p0p + w1p * p1p;
        if (!diry) { S(s->wxR, k, i, j) = vR; S(s->wxL, k, i, j) = vL; }
        else { S(s->wyR, k, i, j) = vR; S(s->wyL, k, i, j) = vL; }
      }
}

/* WENO2D_primvar.cpp:95-198 (beta_1 uses the -2 neighbour, :145,174) */
static void weno5(oracle *o, int nb, int diry, scr_t *s) {
  const double e = 1.E-15;
  for (int i = o->nxminb; i <= o->nxmaxb; i++)
    for (int j = o->nyminb; j <= o->nymaxb; j++)
      for (int k = 0; k < 8; k++) {
        if (!diry && k == 5) continue;
        if (diry && k == 6) continue;
        int di = diry ? 0 : 1, dj = diry ? 1 : 0;
        double w = Qc(o->W, nb, k, i, j);
        double wp = Qc(o->W, nb, k, i + di, j + dj), wpp = Qc(o->W, nb, k, i + 2 * di, j + 2 * dj);
        double wm = Qc(o->W, nb, k, i - di, j - dj), wmm = Qc(o->W, nb, k, i - 2 * di, j - 2 * dj);
        double t;
        double p0n = (-1 * wmm + 5 * wm + 2 * w) / 6;
        double p1n = (2 * wm + 5 * w - wp) / 6;
        double p2n = (11 * w - 7 * wp + 2 * wpp) / 6;
        double t2;
        t = wmm - 2 * wm + w; t2 = wmm - 4 * wm + 3 * w;
        double B0n = (13. / 12.) * (t * t) + (1. / 4.) * (t2 * t2);
        t = wmm - 2 * w + wp; t2 = wm - wp;
        double B1n = (13. / 12.) * (t * t) + (1. / 4.) * (t2 * t2);
        t = w - 2 * wp + wpp; t2 = 3 * w - 4 * wp + wpp;
        double B2n = (13. / 12.) * (t * t) + (1. / 4.) * (t2 * t2);
        double d0n = 1. / 10., d1n = 6. / 10., d2n = 3. / 10.;
        double a0n = d0n / ((e + B0n) * (e + B0n));
        double a1n = d1n / ((e + B1n) * (e + B1n));
        double a2n = d2n / ((e + B2n) * (e + B2n));
        double asn = a0n + a1n + a2n;
        double w0n = a0n / asn, w1n = a1n / asn, w2n = a2n / asn;
        double vR = w0n * p0n + w1n * p1n + w2n * p2n;
        double p0p = (2 * wmm - 7 * wm + 11 * w) / 6;
        double p1p = (-1 * wm + 5 * w + 2 * wp) / 6;
        double p2p = (2 * w + 5 * wp - wpp) / 6;
        t = wmm - 2 * wm + w; t2 = wmm - 4 * wm + 3 * w;
        double B0p = (13. / 12.) * (t * t) + (1. / 4.) * (t2 * t2);
        t = wmm - 2 * w + wp; t2 = wm - wp;
        double B1p = (13. / 12.) * (t * t) + (1. / 4.) * (t2 * t2);
        t = w - 2 * wp + wpp; t2 = 3 * w - 4 * wp + wpp;
        double B2p = (13. / 12.) * (t * t) + (1. / 4.) * (t2 * t2);
        double d0p = 3. / 10., d1p = 6. / 10., d2p = 1. / 10.;
        double a0p = d0p / ((e + B0p) * (e + B0p));
        double a1p = d1p / ((e + B1p) * (e + B1p));
        double a2p = d2p / ((e + B2p) * (e + B2p));
        double asp = a0p + a1p + a2p;
        double w0p = a0p / asp, w1p = a1p / asp, w2p = a2p / asp;
        double vL = w0p * p0p + w1p * p1p + w2p * p2p;
        if (!diry) { S(s->wxR, k, i, j) = vR; S(s->wxL, k, i, j) = vL; }
        else { S(s->wyR, k, i, j) = vR; S(s->wyL, k, i, j) = vL; }
      }
}

/* ------------------------------------------------------------ MUSCL2D.cpp */
/* MUSCL2D.cpp:13-121 followed by the residual / RK2ndv1 loop of
 * main.cpp:147-157 (step 1) or main.cpp:179-189 (step 2). */
static int muscl_rk(oracle *o, int nb, int step) {
  scr_t s = thread_scratch(o);
  if (cons2prim(o, step == 1 ? o->U : o->Us, nb, step == 2)) return -1;
  if (o->c.limiter == OR_LIM_WENO3) { weno3(o, nb, 0, &s); weno3(o, nb, 1, &s); }
  else if (o->c.limiter == OR_LIM_WENO5) { weno5(o, nb, 0, &s); weno5(o, nb, 1, &s); }
  else if (celledges(o, nb, &s)) return -1;
  const double *B = step == 1 ? o->Bi : o->Bis;
  for (int i = 0; i < o->nx - 1; i++)      /* MUSCL2D.cpp:44-53 */
    for (int j = 0; j < o->ny - 1; j++) {
      S(s.wxL, 5, i, j) = Qf(B, nb, 0, i + 1, j);
      S(s.wxR, 5, i, j) = Qf(B, nb, 0, i, j);
      S(s.wyL, 6, i, j) = Qf(B, nb, 1, i, j + 1);
      S(s.wyR, 6, i, j) = Qf(B, nb, 1, i, j);
    }
  for (int i = o->nxminb; i <= o->nxmax; i++)   /* MUSCL2D.cpp:63-116 */
    for (int j = o->nyminb; j <= o->nymax; j++) {
      double wL[8], wR[8], f[8];
      for (int k = 0; k < 8; k++) { wL[k] = S(s.wxL, k, i, j); wR[k] = S(s.wxR, k, i + 1, j); }
      int rc = oracle_riemann(o->c.flux, wL, wR, o->gamma, 0, f);
      if (rc) return fail(o, rc == -4 ? "ROE not ready with magnetic field" : "HLLC trap");
      for (int k = 0; k < 8; k++) {
        Qc(o->ff, nb, k, i + 1, j) = f[k];
        if (isnan(f[k])) return fail(o, "NaN x-flux");
      }
      for (int k = 0; k < 8; k++) { wL[k] = S(s.wyL, k, i, j); wR[k] = S(s.wyR, k, i, j + 1); }
      rc = oracle_riemann(o->c.flux, wL, wR, o->gamma, 1, f);
      if (rc) return fail(o, rc == -4 ? "ROE not ready with magnetic field" : "HLLC trap");
      for (int k = 0; k < 8; k++) {
        Qc(o->gg, nb, k, i, j + 1) = f[k];
        if (isnan(f[k])) return fail(o, "NaN y-flux");
      }
    }
  double dx = o->dx[o->lp[nb][0]], dy = o->dy[o->lp[nb][0]], dt = o->dt;
  for (int i = 0; i < o->nx; i++)
    for (int j = 0; j < o->ny; j++)
      for (int k = 0; k < 8; k++) {
        double res;
        if ((i >= o->nxminb && i <= o->nxmax) && (j >= o->nyminb && j <= o->nymax))
          res = (Qc(o->ff, nb, k, i + 1, j) - Qc(o->ff, nb, k, i, j)) / dx +
                (Qc(o->gg, nb, k, i, j + 1) - Qc(o->gg, nb, k, i, j)) / dy;
        else res = 0.;
        /* timeIntegral.cpp:3-9 */
        if (step == 1) Qc(o->Us, nb, k, i, j) = Qc(o->U, nb, k, i, j) - dt * res;
        else Qc(o->U, nb, k, i, j) = 0.5 * (Qc(o->U, nb, k, i, j) + Qc(o->Us, nb, k, i, j) - dt * res);
      }
  return 0;
}

/* ------------------------------------------- boundary*.cpp, extboundary */
/* The fine-to-coarse operator of the three ghost fills:
 *   cell centred  boundary.cpp:48-49     0.25 * sum of a 2x2 patch
 *   face centred  boundaryfc.cpp:48-51   0.5 * sum of two faces along the
 *                                        face's own direction (k==0: j, j+1)
 *   edge centred  boundaryec.cpp:46-47   injection of one value             */
static inline double fine_val(const oracle *o, const fld *f, int nb, int k, int i1, int j1) {
  if (f->kind == K_EC) return F(f, nb, k, i1, j1);
  int i2, j2;
  double c;
  if (f->kind == K_CC) { i2 = i1 + 1; j2 = j1 + 1; c = 0.25; }
  else { i2 = k == 0 ? i1 : i1 + 1; j2 = k == 0 ? j1 + 1 : j1; c = 0.5; }
  double v = 0.;                 /* misc.cpp:23-37 sum_irjr */
  for (int i = i1; i <= i2; i++)
    for (int j = j1; j <= j2; j++) v += F(f, nb, k, i, j);
  return c * v;
}

/* extboundary.cpp:5-61 */
static void extboundary(oracle *o, fld *f) {
  int ng = o->ng, nv = f->nv;
  for (int b = 0; b < o->nbounds; b++) {
    int nbs = o->ib[b][0];
    int ii, jj;
    switch (o->ib[b][2]) {
      case -1:
        ii = o->nxmin + (ng - 1);
        for (int i = 0; i < ng; i++) {
          for (int j = 0; j < o->ny; j++)
            for (int k = 0; k < nv; k++) F(f, nbs, k, i, j) = F(f, nbs, k, ii, j);
          ii--;
        }
        break;
      case -2:
        ii = o->nxmax;
        for (int i = o->nxp1; i < o->nx; i++) {
          for (int j = 0; j < o->ny; j++)
            for (int k = 0; k < nv; k++) F(f, nbs, k, i, j) = F(f, nbs, k, ii, j);
          ii--;
        }
        break;
      case -3:
        jj = o->nymin + (ng - 1);
        for (int j = 0; j < ng; j++) {
          for (int i = 0; i < o->nx; i++)
            for (int k = 0; k < nv; k++) F(f, nbs, k, i, j) = F(f, nbs, k, i, jj);
          jj--;
        }
        break;
      case -4:
        jj = o->nymax;
        for (int j = o->nyp1; j < o->ny; j++) {
          for (int i = 0; i < o->nx; i++)
            for (int k = 0; k < nv; k++) F(f, nbs, k, i, j) = F(f, nbs, k, i, jj);
          jj--;
        }
        break;
      default: break;
    }
  }
}

/* boundary.cpp:7-388 / boundaryfc.cpp:8-404 / boundaryec.cpp:7-378: the three
 * files share their index arithmetic and differ only in fine_val (above). */
static void ghostfill(oracle *o, fld *f) {
  int ng = o->ng, nv = f->nv, nx = o->nx, ny = o->ny;
  int (*lp)[8] = o->lp;
  const int nxmin = o->nxmin, nxmax = o->nxmax, nymin = o->nymin, nymax = o->nymax;
  const int nxminb = o->nxminb, nxmaxb = o->nxmaxb, nyminb = o->nyminb, nymaxb = o->nymaxb;
  const int nxp1 = o->nxp1, nyp1 = o->nyp1, nx2 = o->nx2, ny2 = o->ny2;
  for (int b = 0; b < o->nbounds; b++) {
    int nbs = o->ib[b][0], n1, n2, n3, n4, ii, jj;
    switch (o->ib[b][2]) {
      case 1: /* boundary.cpp:17-35 */
        n1 = o->ib[b][1];
        for (int j = 0; j < ny; j++)
          for (int k = 0; k < nv; k++) {
            ii = nxmax - (ng - 1);
            for (int i = 0; i < ng; i++) { F(f, nbs, k, i, j) = F(f, n1, k, ii, j); ii++; }
            ii = nxmin;
            for (int i = nxp1; i < nx; i++) { F(f, n1, k, i, j) = F(f, nbs, k, ii, j); ii++; }
          }
        break;
      case 2: /* boundary.cpp:36-107 */
        n1 = o->ib[b][1];
        n2 = n1 + 2;
        for (int j = nymin; j <= ny2; j++) {
          int ny2j = ny2 + j - 1 - (ng - 2);
          for (int i = 0; i < ng; i++) {
            int i1 = 2 * (i - ng / 2) - ng / 2 + nxmax, j1 = 2 * j - nymin;
            for (int k = 0; k < nv; k++) {
              F(f, nbs, k, i, j) = fine_val(o, f, n1, k, i1, j1);
              F(f, nbs, k, i, ny2j) = fine_val(o, f, n2, k, i1, j1);
            }
          }
        }
        n3 = lp[lp[n1][1]][6];
        if (n3 != -1) {
          if (o->leafs[n3]) {
            for (int k = 0; k < nv; k++)
              for (int i = 0; i < ng; i++)
                for (int j = 0; j < ng; j++) {
                  ii = nxmax - ng + (i + 1); jj = nymax - ng + (j + 1);
                  F(f, nbs, k, i, j) = F(f, n3, k, ii, jj);
                }
          } else {
            n3 = lp[n3][2] + 3;
            if (o->leafs[n3])
              for (int k = 0; k < nv; k++)
                for (int i = 0; i < ng; i++)
                  for (int j = 0; j < ng; j++) {
                    ii = nxmax - ng * 2 + 2 * i + 1; jj = nymax - ng * 2 + 2 * j + 1;
                    F(f, nbs, k, i, j) = fine_val(o, f, n3, k, ii, jj);
                  }
          }
        }
        n4 = lp[lp[n2][1]][7];
        if (n4 != -1) {
          if (o->leafs[n4]) {
            for (int k = 0; k < nv; k++)
              for (int i = 0; i < ng; i++)
                for (int j = 0; j < ng; j++) {
                  ii = nxmax - ng + (i + 1); jj = nymin + ng - (j + 1);
                  F(f, nbs, k, i, ny - 1 - j) = F(f, n4, k, ii, jj);
                }
          } else {
            n4 = lp[n4][2] + 1;
            if (o->leafs[n4])
              for (int k = 0; k < nv; k++)
                for (int i = 0; i < ng; i++)
                  for (int j = 0; j < ng; j++) {
                    ii = nxmax - ng * 2 + 2 * i + 1; jj = nymin + ng * 2 - 2 * (j + 1);
                    F(f, nbs, k, i, ny - 1 - j) = fine_val(o, f, n4, k, ii, jj);
                  }
          }
        }
        for (int i = 1; i <= ng; i++)
          for (int j = 0; j < ny; j++)
            for (int k = 0; k < nv; k++) {
              F(f, n1, k, i + nxmax, j) = F(f, nbs, k, (i + 2 * ng - 1) / 2, (j + ng) / 2);
              F(f, n2, k, i + nxmax, j) = F(f, nbs, k, (i + 2 * ng - 1) / 2, (j - ng + 2) / 2 + ny2);
            }
        break;
      case 4: /* boundary.cpp:109-127 */
        n1 = o->ib[b][1];
        for (int j = 0; j < ny; j++)
          for (int k = 0; k < nv; k++) {
            ii = nxmin;
            for (int i = nxp1; i < nx; i++) { F(f, nbs, k, i, j) = F(f, n1, k, ii, j); ii++; }
            ii = nxmax - (ng - 1);
            for (int i = 0; i < ng; i++) { F(f, n1, k, i, j) = F(f, nbs, k, ii, j); ii++; }
          }
        break;
      case 5: /* boundary.cpp:128-197 */
        n1 = o->ib[b][1];
        n2 = n1 + 2;
        for (int i = nxp1; i < nx; i++)
          for (int j = nymin; j <= ny2; j++) {
            int i1 = 2 * (i - nxmax + (ng / 2 - 1)), j1 = 2 * j - nymin;
            int ny2j = ny2 + j - 1 - (ng - 2);
            for (int k = 0; k < nv; k++) {
              F(f, nbs, k, i, j) = fine_val(o, f, n1, k, i1, j1);
              F(f, nbs, k, i, ny2j) = fine_val(o, f, n2, k, i1, j1);
            }
          }
        n3 = lp[lp[n1][1]][6];
        if (n3 != -1) {
          if (o->leafs[n3]) {
            for (int k = 0; k < nv; k++)
              for (int i = nxmaxb; i < nx; i++)
                for (int j = 0; j < ng; j++) {
                  ii = nxminb + (i - nxmax); jj = nymax - ng + (j + 1);
                  F(f, nbs, k, i, j) = F(f, n3, k, ii, jj);
                }
          } else {
            n3 = lp[n3][2] + 2;
            if (o->leafs[n3])
              for (int k = 0; k < nv; k++)
                for (int i = nxmaxb; i < nx; i++)
                  for (int j = 0; j < ng; j++) {
                    ii = nxminb + 2 * (i - nxmax) - 1; jj = nymax - ng * 2 + 2 * j + 1;
                    F(f, nbs, k, i, j) = fine_val(o, f, n3, k, ii, jj);
                  }
          }
        }
        n4 = lp[lp[n2][1]][7];
        if (n4 != -1) {
          if (o->leafs[n4]) {
            for (int k = 0; k < nv; k++)
              for (int i = nxmaxb; i < nx; i++)
                for (int j = 0; j < ng; j++) {
                  ii = nxminb + (i - nxmax); jj = nymin + ng - (j + 1);
                  F(f, nbs, k, i, ny - 1 - j) = F(f, n4, k, ii, jj);
                }
          } else {
            n4 = lp[n4][2];
            if (o->leafs[n4])
              for (int k = 0; k < nv; k++)
                for (int i = nxmaxb; i < nx; i++)
                  for (int j = 0; j < ng; j++) {
                    ii = nxminb + 2 * (i - nxmax) - 1; jj = nymin + ng * 2 - 2 * (j + 1);
                    F(f, nbs, k, i, ny - 1 - j) = fine_val(o, f, n4, k, ii, jj);
                  }
          }
        }
        for (int i = 1; i <= ng; i++)
          for (int j = 0; j < ny; j++)
            for (int k = 0; k < nv; k++) {
              F(f, n1, k, i - 1, j) = F(f, nbs, k, (i + 1) / 2 + nxmax - ng / 2, (j + ng) / 2);
              F(f, n2, k, i - 1, j) = F(f, nbs, k, (i + 1) / 2 + nxmax - ng / 2, (j - ng + 2) / 2 + ny2);
            }
        break;
      case 7: /* boundary.cpp:199-217 */
        n1 = o->ib[b][1];
        for (int i = 0; i < nx; i++)
          for (int k = 0; k < nv; k++) {
            jj = nymax - (ng - 1);
            for (int j = 0; j < ng; j++) { F(f, nbs, k, i, j) = F(f, n1, k, i, jj); jj++; }
            jj = nymin;
            for (int j = nyp1; j < ny; j++) { F(f, n1, k, i, j) = F(f, nbs, k, i, jj); jj++; }
          }
        break;
      case 8: /* boundary.cpp:218-287 */
        n1 = o->ib[b][1];
        n2 = n1 + 1;
        for (int i = nxmin; i <= nx2; i++) {
          int nx2i = nx2 + i - 1 - (ng - 2);
          for (int j = 0; j < ng; j++) {
            int i1 = 2 * i - nxmin, j1 = 2 * (j - ng / 2) - ng / 2 + nymax;
            for (int k = 0; k < nv; k++) {
              F(f, nbs, k, i, j) = fine_val(o, f, n1, k, i1, j1);
              F(f, nbs, k, nx2i, j) = fine_val(o, f, n2, k, i1, j1);
            }
          }
        }
        n3 = lp[lp[n1][1]][4];
        if (n3 != -1) {
          if (o->leafs[n3]) {
            for (int k = 0; k < nv; k++)
              for (int i = 0; i < ng; i++)
                for (int j = 0; j < ng; j++) {
                  ii = nxmax - ng + (i + 1); jj = nymax - ng + (j + 1);
                  F(f, nbs, k, i, j) = F(f, n3, k, ii, jj);
                }
          } else {
            n3 = lp[n3][2] + 3;
            if (o->leafs[n3])
              for (int k = 0; k < nv; k++)
                for (int i = 0; i < ng; i++)
                  for (int j = 0; j < ng; j++) {
                    ii = nxmax - ng * 2 + 2 * i + 1; jj = nymax - ng * 2 + 2 * j + 1;
                    F(f, nbs, k, i, j) = fine_val(o, f, n3, k, ii, jj);
                  }
          }
        }
        n4 = lp[lp[n2][1]][5];
        if (n4 != -1) {
          if (o->leafs[n4]) {
            for (int k = 0; k < nv; k++)
              for (int i = 0; i < ng; i++)
                for (int j = 0; j < ng; j++) {
                  ii = nxmin + ng - (i + 1); jj = nymax - ng + (j + 1);
                  F(f, nbs, k, nx - 1 - i, j) = F(f, n4, k, ii, jj);
                }
          } else {
            n4 = lp[n4][2] + 2;
            if (o->leafs[n4])
              for (int k = 0; k < nv; k++)
                for (int i = 0; i < ng; i++)
                  for (int j = 0; j < ng; j++) {
                    ii = nxmin + ng * 2 - 2 * (i + 1); jj = nymax - ng * 2 + 2 * j + 1;
                    F(f, nbs, k, nx - 1 - i, j) = fine_val(o, f, n4, k, ii, jj);
                  }
          }
        }
        for (int j = 1; j <= ng; j++)
          for (int i = 0; i < nx; i++)
            for (int k = 0; k < nv; k++) {
              F(f, n1, k, i, j + nymax) = F(f, nbs, k, (i + ng) / 2, (j + 2 * ng - 1) / 2);
              F(f, n2, k, i, j + nymax) = F(f, nbs, k, (i - ng + 2) / 2 + nx2, (j + 2 * ng - 1) / 2);
            }
        break;
      case 10: /* boundary.cpp:289-307 */
        n1 = o->ib[b][1];
        for (int i = 0; i < nx; i++)
          for (int k = 0; k < nv; k++) {
            jj = nymin;
            for (int j = nyp1; j < ny; j++) { F(f, nbs, k, i, j) = F(f, n1, k, i, jj); jj++; }
            jj = nymax - (ng - 1);
            for (int j = 0; j < ng; j++) { F(f, n1, k, i, j) = F(f, nbs, k, i, jj); jj++; }
          }
        break;
      case 11: /* boundary.cpp:308-377 */
        n1 = o->ib[b][1];
        n2 = n1 + 1;
        for (int i = nxmin; i <= nx2; i++)
          for (int j = nyp1; j < ny; j++) {
            int i1 = 2 * i - nxmin, j1 = 2 * (j - nymax + (ng / 2 - 1));
            int nx2i = nx2 + i - 1 - (ng - 2);
            for (int k = 0; k < nv; k++) {
              F(f, nbs, k, i, j) = fine_val(o, f, n1, k, i1, j1);
              F(f, nbs, k, nx2i, j) = fine_val(o, f, n2, k, i1, j1);
            }
          }
        n3 = lp[lp[n1][1]][4];
        if (n3 != -1) {
          if (o->leafs[n3]) {
            for (int k = 0; k < nv; k++)
              for (int i = 0; i < ng; i++)
                for (int j = nymaxb; j < ny; j++) {
                  ii = nxmax - ng + (i + 1); jj = nyminb + (j - nymax);
                  F(f, nbs, k, i, j) = F(f, n3, k, ii, jj);
                }
          } else {
            n3 = lp[n3][2] + 1;
            if (o->leafs[n3])
              for (int k = 0; k < nv; k++)
                for (int i = 0; i < ng; i++)
                  for (int j = nymaxb; j < ny; j++) {
                    ii = nxmax - ng * 2 + 2 * i + 1; jj = nyminb + 2 * (j - nymax) - 1;
                    F(f, nbs, k, i, j) = fine_val(o, f, n3, k, ii, jj);
                  }
          }
        }
        n4 = lp[lp[n2][1]][5];
        if (n4 != -1) {
          if (o->leafs[n4]) {
            /* boundary.cpp:348-354 and boundaryfc.cpp:362-368 walk this
             * corner in different orders onto the same cells */
            for (int k = 0; k < nv; k++)
              for (int i = 0; i < ng; i++)
                for (int j = nymaxb; j < ny; j++) {
                  ii = nxmin + ng - (i + 1); jj = nyminb + (j - nymax);
                  F(f, nbs, k, nx - 1 - i, j) = F(f, n4, k, ii, jj);
                }
          } else {
            n4 = lp[n4][2];
            if (o->leafs[n4])
              for (int k = 0; k < nv; k++)
                for (int i = nxmaxb; i < nx; i++)
                  for (int j = nymaxb; j < ny; j++) {
                    ii = nxminb + 2 * (i - nxmax) - 1; jj = nyminb + 2 * (j - nymax) - 1;
                    F(f, nbs, k, i, j) = fine_val(o, f, n4, k, ii, jj);
                  }
          }
        }
        for (int j = 1; j <= ng; j++)
          for (int i = 0; i < nx; i++)
            for (int k = 0; k < nv; k++) {
              F(f, n1, k, i, j - 1) = F(f, nbs, k, (i + ng) / 2, (j + 1) / 2 + nymax - ng / 2);
              F(f, n2, k, i, j - 1) = F(f, nbs, k, (i - ng + 2) / 2 + nx2, (j + 1) / 2 + nymax - ng / 2);
            }
        break;
      default: break;
    }
  }
  extboundary(o, f);
}

static void fill_cc(oracle *o, double *a) { fld f = {a, 8, K_CC}; ghostfill(o, &f); }
static void fill_fc(oracle *o, double *a, int nv) { fld f = {a, nv, K_FC}; ghostfill(o, &f); }
static void fill_ec(oracle *o, double *a) { fld f = {a, 1, K_EC}; ghostfill(o, &f); }

/* --------------------------------------------------------- locate_bounds */
static void add_bound(oracle *o, int s, int d, int c) {
  int n = o->nbounds++;
  o->ib[n][0] = s; o->ib[n][1] = d; o->ib[n][2] = c;
}

/* locate_bounds.cpp:35-208 */
static void locate_bounds(oracle *o) {
  int (*lp)[8] = o->lp;
  unsigned char (*bd)[4] = (unsigned char (*)[4])o->bflag;
  memset(o->bflag, 0, (size_t)4 * o->maxblocks);
  o->nbounds = 0;
  for (int nb = 0; nb < o->lastActive; nb++) {
    if (!o->leafs[nb]) continue;
    int n1, n2;
    if (!bd[nb][0]) {
      if (lp[nb][4] == -1) { bd[nb][0] = 1; add_bound(o, nb, -1, -1); }
      else if (lp[lp[nb][4]][0] >= lp[nb][0]) {
        n1 = lp[nb][4];
        if (o->leafs[n1]) { add_bound(o, nb, n1, 1); bd[nb][0] = 1; bd[n1][1] = 1; }
        else {
          bd[nb][0] = 1;
          n1 = lp[n1][2] + 1; n2 = n1 + 2;
          add_bound(o, nb, n1, 2);
          bd[n1][1] = 1; bd[n2][1] = 1;
        }
      }
    }
    if (!bd[nb][1]) {
      if (lp[nb][5] == -1) { bd[nb][1] = 1; add_bound(o, nb, -1, -2); }
      else if (lp[lp[nb][5]][0] >= lp[nb][0]) {
        n1 = lp[nb][5];
        if (o->leafs[n1]) { add_bound(o, nb, n1, 4); bd[nb][1] = 1; bd[n1][0] = 1; }
        else {
          bd[nb][1] = 1;
          n1 = lp[n1][2]; n2 = n1 + 2;
          add_bound(o, nb, n1, 5);
          bd[n1][0] = 1; bd[n2][0] = 1;
        }
      }
    }
    if (!bd[nb][2]) {
      if (lp[nb][6] == -1) { bd[nb][2] = 1; add_bound(o, nb, -1, -3); }
      else if (lp[lp[nb][6]][0] >= lp[nb][0]) {
        n1 = lp[nb][6];
        if (o->leafs[n1]) { add_bound(o, nb, n1, 7); bd[nb][2] = 1; bd[n1][3] = 1; }
        else {
          bd[nb][2] = 1;
          n1 = lp[n1][2] + 2; n2 = n1 + 1;
          add_bound(o, nb, n1, 8);
          bd[n1][3] = 1; bd[n2][3] = 1;
        }
      }
    }
    if (!bd[nb][3]) {
      if (lp[nb][7] == -1) { bd[nb][3] = 1; add_bound(o, nb, -1, -4); }
      else if (lp[lp[nb][7]][0] >= lp[nb][0]) {
        n1 = lp[nb][7];
        if (o->leafs[n1]) { add_bound(o, nb, n1, 10); bd[nb][3] = 1; bd[n1][2] = 1; }
        else {
          bd[nb][3] = 1;
          n1 = lp[n1][2]; n2 = n1 + 1;
          add_bound(o, nb, n1, 11);
          bd[n1][2] = 1; bd[n2][2] = 1;
        }
      }
    }
  }
}

/* diffusivity.cpp:6-17 on one block (main.cpp:190-193 applies it after the
 * stage-2 update of every leaf at level >= maxlevs - 2 when `diffusion` is
 * on): U += eta * (5-point Laplacian) over the interior, in place with i
 * outer and j inner, so a cell sees the new values of its (i-1, j) and
 * (i, j-1) neighbours; eta = 0.001 (defs.hpp:50). */
static void diffuse(oracle *o, double *U, int nb) {
  const double eta = 0.001;
  for (int i = o->nxmin; i <= o->nxmax; i++)
    for (int j = o->nymin; j <= o->nymax; j++)
      for (int k = 0; k < 8; k++)
        Qc(U, nb, k, i, j) = Qc(U, nb, k, i, j) + eta * (Qc(U, nb, k, i + 1, j) + Qc(U, nb, k, i - 1, j) +
                                                         Qc(U, nb, k, i, j + 1) + Qc(U, nb, k, i, j - 1) -
                                                         4. * Qc(U, nb, k, i, j));
}

/* ---------------------------------------------------------------- CT2D.cpp */
/* CT2D.cpp:28-75, CTtype == 2 ("upwind (not ready)", defs.hpp:34) for one
 * block: pressure p and speed C of every cell of q (:36-40), then the corner
 * EMF weighting the two flux averages by psi, which leaves 1/2 unless the
 * corner sits at a strong pressure jump (switch 1, beta = 0.5) in a strongly
 * compressive flow (switch 2, delta = 0.1).  The divergence term divides
 * rho*v by itself at two of its corners (:52), as the reference does.
 * Returns 1 on the reference's "Incorrect psi produced" (:68). */
static int emf_upwind(oracle *o, const double *q, int nb) {
  const int nx = o->nx, ny = o->ny;
  const double g = o->gamma;
  double *p = (double *)malloc(sizeof(double) * 2 * nx * ny), *C = p + nx * ny;
  int bad = 0;
#define PC(A, i, j) (A)[(j) * nx + (i)]
  for (int i = 0; i < nx; i++)
    for (int j = 0; j < ny; j++) {
      double q0 = Qc(q, nb, 0, i, j), q1 = Qc(q, nb, 1, i, j), q2 = Qc(q, nb, 2, i, j), q3 = Qc(q, nb, 3, i, j);
      double q4 = Qc(q, nb, 4, i, j), q5 = Qc(q, nb, 5, i, j), q6 = Qc(q, nb, 6, i, j), q7 = Qc(q, nb, 7, i, j);
      PC(p, i, j) = (g - 1) * (q4 - 0.5 * ((q1 * q1 + q2 * q2 + q3 * q3) / q0 + (q5 * q5 + q6 * q6 + q7 * q7)));
      PC(C, i, j) = sqrt((g * PC(p, i, j) + (q5 * q5 + q6 * q6 + q7 * q7)) / q0);
    }
  for (int i = 1; i < nx; i++)
    for (int j = 1; j < ny; j++) {
      const double beta = 0.5, delta = 0.1;
      double dPx = 0.5 * fabs(PC(p, i, j) + PC(p, i, j - 1) - PC(p, i - 1, j) - PC(p, i - 1, j - 1));
      double dPy = 0.5 * fabs(PC(p, i, j) + PC(p, i - 1, j) - PC(p, i, j - 1) - PC(p, i - 1, j - 1));
      double divV = 0.5 * (Qc(q, nb, 1, i, j) / Qc(q, nb, 0, i, j) + Qc(q, nb, 1, i, j - 1) / Qc(q, nb, 0, i, j - 1) -
                           Qc(q, nb, 1, i - 1, j) / Qc(q, nb, 0, i - 1, j) -
                           Qc(q, nb, 1, i - 1, j - 1) / Qc(q, nb, 0, i - 1, j - 1)) +
                    0.5 * (Qc(q, nb, 2, i, j) / Qc(q, nb, 0, i, j) + Qc(q, nb, 2, i - 1, j) / Qc(q, nb, 2, i - 1, j) -
                           Qc(q, nb, 2, i, j - 1) / Qc(q, nb, 2, i, j - 1) -
                           Qc(q, nb, 2, i - 1, j - 1) / Qc(q, nb, 0, i - 1, j - 1));
      double tempP = MMIN(PC(p, i - 1, j - 1), PC(p, i, j - 1));
      double tempP1 = MMIN(PC(p, i - 1, j), PC(p, i, j));
      tempP = MMIN(tempP, tempP1);
      int sw1 = (dPx + dPy) > beta * tempP;
      double tempC = MMIN(PC(C, i - 1, j - 1), PC(C, i, j - 1));
      double tempC1 = MMIN(PC(C, i - 1, j), PC(C, i, j));
      tempC = MMIN(tempC, tempC1);
      int sw2 = (-delta * tempC) > divV;
      double psi = 0.5;
      if (sw1 && sw2) psi = dPx / (dPx + dPy);
      if (psi < 0 || psi > 1) bad = 1;
      Qe(o->EMF, nb, i, j) = 0.5 * (1. - psi) * (Qc(o->gg, nb, 5, i - 1, j) + Qc(o->gg, nb, 5, i, j)) -
                             0.5 * psi * (Qc(o->ff, nb, 6, i, j - 1) + Qc(o->ff, nb, 6, i, j));
    }
#undef PC
  free(p);
  return bad;
}

/* CT2D.cpp:11-124.  q is the cell state being corrected, Bi the face field
 * at the start of the stage, Binew the output. */
static int ct2d(oracle *o, double *q, double *Bi, int step, double *Binew) {
  int nL = 0;
  int *leaf = (int *)malloc(sizeof(int) * (o->lastActive + 1));
  for (int nb = 0; nb < o->lastActive; nb++) if (o->leafs[nb]) leaf[nL++] = nb;
  int bad = 0;
#pragma omp parallel for schedule(static) num_threads(o->nthreads) reduction(| : bad)
  for (int l = 0; l < nL; l++) {
    int nb = leaf[l];
    if (o->c.ct_type == 2) {
      bad |= emf_upwind(o, q, nb);
      continue;
    }
    for (int i = 1; i < o->nx; i++)
      for (int j = 1; j < o->ny; j++)
        Qe(o->EMF, nb, i, j) = 0.25 * ((Qc(o->gg, nb, 5, i - 1, j) + Qc(o->gg, nb, 5, i, j)) -
                                       (Qc(o->ff, nb, 6, i, j - 1) + Qc(o->ff, nb, 6, i, j)));
  }
  if (bad) { free(leaf); return fail(o, "Incorrect psi produced"); }
  fill_ec(o, o->EMF);
  double dt = o->dt;
#pragma omp parallel for schedule(static) num_threads(o->nthreads)
  for (int l = 0; l < nL; l++) {
    int nb = leaf[l];
    double dx = o->dx[o->lp[nb][0]], dy = o->dy[o->lp[nb][0]];
    for (int i = 0; i < o->nx; i++)
      for (int j = 0; j < o->ny; j++) {
        int ip = i < o->nx - 1 ? i + 1 : i, jp = j < o->ny - 1 ? j + 1 : j;
        double res = (1. / dy) * (Qe(o->EMF, nb, i, jp) - Qe(o->EMF, nb, i, j));
        if (step == 1) Qf(Binew, nb, 0, i, j) = Qf(Bi, nb, 0, i, j) - dt * res;
        else Qf(Binew, nb, 0, i, j) = 0.5 * (Qf(Bi, nb, 0, i, j) + Qf(Binew, nb, 0, i, j) - dt * res);
        res = -(1. / dx) * (Qe(o->EMF, nb, ip, j) - Qe(o->EMF, nb, i, j));
        if (step == 1) Qf(Binew, nb, 1, i, j) = Qf(Bi, nb, 1, i, j) - dt * res;
        else Qf(Binew, nb, 1, i, j) = 0.5 * (Qf(Bi, nb, 1, i, j) + Qf(Binew, nb, 1, i, j) - dt * res);
      }
  }
  fill_fc(o, Binew, 2);
#pragma omp parallel for schedule(static) num_threads(o->nthreads)
  for (int l = 0; l < nL; l++) {
    int nb = leaf[l];
    for (int i = 0; i < o->nx; i++)
      for (int j = 0; j < o->ny; j++) {
        int ip = i < o->nx - 1 ? i + 1 : i, ii = ip - 1;
        int jp = j < o->ny - 1 ? j + 1 : j, jj = jp - 1;
        double Bx = 0.5 * (Qf(Binew, nb, 0, ip, j) + Qf(Binew, nb, 0, ii, j));
        double By = 0.5 * (Qf(Binew, nb, 1, i, jp) + Qf(Binew, nb, 1, i, jj));
        double q5 = Qc(q, nb, 5, i, j), q6 = Qc(q, nb, 6, i, j);
        Qc(q, nb, 4, i, j) = Qc(q, nb, 4, i, j) + 0.5 * ((Bx * Bx + By * By) - (q5 * q5 + q6 * q6));
        Qc(q, nb, 5, i, j) = Bx;
        Qc(q, nb, 6, i, j) = By;
      }
  }
  free(leaf);
  return 0;
}

/* ------------------------------------------------------- refine / coarsen */
/* refine.cpp:17-36 (rlimiter = "minmod", defs.hpp:36) */
static double refine_sl(oracle *o, const double *Q, int i, int j, int k, int nb, int sx, int sy) {
  double result = Qc(Q, nb, k, i, j), r, phi;
  r = (Qc(Q, nb, k, i, j) - Qc(Q, nb, k, i - 1, j)) / (Qc(Q, nb, k, i + 1, j) - Qc(Q, nb, k, i, j) + EPS);
  phi = 0.25 * oracle_slopelimiter(OR_LIM_MINMOD, r, 0) * (Qc(Q, nb, k, i + 1, j) - Qc(Q, nb, k, i, j));
  result = sx == 0 ? result - phi : result + phi;
  r = (Qc(Q, nb, k, i, j) - Qc(Q, nb, k, i, j - 1)) / (Qc(Q, nb, k, i, j + 1) - Qc(Q, nb, k, i, j) + EPS);
  phi = 0.25 * oracle_slopelimiter(OR_LIM_MINMOD, r, 0) * (Qc(Q, nb, k, i, j + 1) - Qc(Q, nb, k, i, j));
  result = sy == 0 ? result - phi : result + phi;
  return result;
}

/* refine.cpp:38-85 */
static int refine(oracle *o, int nb, const int *son) {
  int ng = o->ng;
  for (int i = 0; i < o->nx; i++)
    for (int j = 0; j < o->ny; j++)
      for (int k = 0; k < 8; k++) {
        int sx = (i + ng) % 2, sy = (j + ng) % 2;
        int ii = (i + ng) / 2, jj = (j + ng) / 2;
        Qc(o->U, son[0], k, i, j) = refine_sl(o, o->U, ii, jj, k, nb, sx, sy);
        ii = (i - ng + 2) / 2 + o->nx2;
        Qc(o->U, son[1], k, i, j) = refine_sl(o, o->U, ii, jj, k, nb, sx, sy);
        ii = (i + ng) / 2; jj = (j - ng + 2) / 2 + o->ny2;
        Qc(o->U, son[2], k, i, j) = refine_sl(o, o->U, ii, jj, k, nb, sx, sy);
        ii = (i - ng + 2) / 2 + o->nx2;
        Qc(o->U, son[3], k, i, j) = refine_sl(o, o->U, ii, jj, k, nb, sx, sy);
      }
  int nx0 = o->icoord[nb][0] * 2, ny0 = o->icoord[nb][1] * 2;
  int ni = o->nx - 2 * ng, nj = o->ny - 2 * ng;
  const int off[4][2] = {{0, 0}, {ni, 0}, {0, nj}, {ni, nj}};
  for (int s = 0; s < 4; s++) {
    if (cons2prim(o, o->U, son[s], 0)) return -1;
    o->icoord[son[s]][0] = nx0 + off[s][0];
    o->icoord[son[s]][1] = ny0 + off[s][1];
  }
  return 0;
}

/* refineBi_CT.cpp:4-50 */
static double refine_sl_bi(oracle *o, const double *B, int i, int j, int k, int nb, int sx, int sy) {
  double Bx_jm = Qf(B, nb, 0, i, j - 1), Bx = Qf(B, nb, 0, i, j), Bx_jp = Qf(B, nb, 0, i, j + 1);
  double Bx_ip = Qf(B, nb, 0, i + 1, j), Bx_ipjm = Qf(B, nb, 0, i + 1, j - 1),
         Bx_ipjp = Qf(B, nb, 0, i + 1, j + 1);
  double By_im = Qf(B, nb, 1, i - 1, j), By = Qf(B, nb, 1, i, j), By_ip = Qf(B, nb, 1, i + 1, j);
  double By_imjp = Qf(B, nb, 1, i - 1, j + 1), By_jp = Qf(B, nb, 1, i, j + 1),
         By_ipjp = Qf(B, nb, 1, i + 1, j + 1);
  double r;
  r = (Bx - Bx_jm) / (Bx_jp - Bx + EPS);
  double DyBxm = oracle_slopelimiter(OR_LIM_MINMOD, r, 0) * (Bx_jp - Bx);
  r = (Bx_ip - Bx_ipjm) / (Bx_ipjp - Bx_ip + EPS);
  double DyBxp = oracle_slopelimiter(OR_LIM_MINMOD, r, 0) * (Bx_ipjp - Bx_ip);
  r = (By - By_im) / (By_ip - By + EPS);
  double DxBym = oracle_slopelimiter(OR_LIM_MINMOD, r, 0) * (By_ip - By);
  r = (By_jp - By_imjp) / (By_ipjp - By_jp + EPS);
  double DxByp = oracle_slopelimiter(OR_LIM_MINMOD, r, 0) * (By_ipjp - By_jp);
  double ax = (Bx_ip - Bx);
  double by = -1. * ax;
  double ay = 0.5 * (DyBxp + DyBxm);
  double bx = 0.5 * (DxByp + DxBym);
  double axy = (DyBxp - DyBxm);
  double byy = axy / (-2.);
  double bxy = (DxByp - DxBym);
  double axx = bxy / (-2.);
  double a0 = 0.5 * (Bx_ip + Bx) - 0.25 * axx;
  double b0 = 0.5 * (By_jp + By) - 0.25 * byy;
  double ayy = 0., bxx = 0.;
  double res;
  if (k == 0) {
    double tx = sx == 0 ? 0 : 0.5, ty = sy == 0 ? -0.25 : 0.25;
    res = a0 + ax * tx + ay * ty + axx * tx * tx + axy * tx * ty + ayy * ty * ty;
  } else {
    double tx = sx == 0 ? -0.25 : 0.25, ty = sy == 0 ? 0 : 0.5;
    res = b0 + bx * tx + by * ty + bxx * tx * tx + bxy * tx * ty + byy * ty * ty;
  }
  return res;
}

/* refineBi_CT.cpp:52-74 */
static int refine_bi(oracle *o, int nb, const int *son) {
  int ng = o->ng;
  for (int i = 0; i < o->nx; i++)
    for (int j = 0; j < o->ny; j++)
      for (int k = 0; k < 2; k++) {
        int sx = (i + ng) % 2, sy = (j + ng) % 2;
        int ii = (i + ng) / 2, jj = (j + ng) / 2;
        double v[4];
        v[0] = refine_sl_bi(o, o->Bi, ii, jj, k, nb, sx, sy);
        ii = (i - ng + 2) / 2 + o->nx2;
        v[1] = refine_sl_bi(o, o->Bi, ii, jj, k, nb, sx, sy);
        ii = (i + ng) / 2; jj = (j - ng + 2) / 2 + o->ny2;
        v[2] = refine_sl_bi(o, o->Bi, ii, jj, k, nb, sx, sy);
        ii = (i - ng + 2) / 2 + o->nx2;
        v[3] = refine_sl_bi(o, o->Bi, ii, jj, k, nb, sx, sy);
        for (int s = 0; s < 4; s++) {
          if (isnan(v[s])) return fail(o, "NaN in face-B prolongation");
          Qf(o->Bi, son[s], k, i, j) = v[s];
        }
      }
  return 0;
}

static inline double sum4(const oracle *o, const double *Q, int nv, int nb, int k, int i1, int i2,
                          int j1, int j2) { /* misc.cpp:23-37 */
  double v = 0.;
  for (int i = i1; i <= i2; i++)
    for (int j = j1; j <= j2; j++) v += Q[IX(o, nb, nv, k, i, j)];
  return v;
}

/* coarsen.cpp:7-157 (U, cell averages) and coarsenBi_CT.cpp:7-155 (face B):
 * face = 1 selects the face form, whose pair along the face direction is
 * (i1, j1..j1+1) for k==0 and (i1..i1+1, j1) otherwise. */
static void coarsen_field(oracle *o, double *Q, int nv, int face, int dad, const int *son) {
  const int ng = o->ng, nx = o->nx, ny = o->ny;
  const int nxmin = o->nxmin, nymin = o->nymin, nxminb = o->nxminb, nyminb = o->nyminb;
  const int nxmaxb = o->nxmaxb, nymaxb = o->nymaxb, nx2 = o->nx2, ny2 = o->ny2;
  const double c = face ? 0.5 : 0.25;
#define I2(k, i1) (face ? ((k) == 0 ? (i1) : (i1) + 1) : (i1) + 1)
#define J2(k, j1) (face ? ((k) == 0 ? (j1) + 1 : (j1)) : (j1) + 1)
#define SUM(nbq, k, i1, j1) (c * sum4(o, Q, nv, nbq, k, i1, I2(k, i1), j1, J2(k, j1)))
  for (int i = nxmin; i <= nx2; i++)
    for (int j = nymin; j <= ny2; j++) {
      int i1 = 2 * i - nxmin, j1 = 2 * j - nymin;
      int nx2i = nx2 + i - 1 - (ng - 2), ny2j = ny2 + j - 1 - (ng - 2);
      for (int k = 0; k < nv; k++) {
        Q[IX(o, dad, nv, k, i, j)] = SUM(son[0], k, i1, j1);
        Q[IX(o, dad, nv, k, nx2i, j)] = SUM(son[1], k, i1, j1);
        Q[IX(o, dad, nv, k, i, ny2j)] = SUM(son[2], k, i1, j1);
        Q[IX(o, dad, nv, k, nx2i, ny2j)] = SUM(son[3], k, i1, j1);
      }
    }
  /* ghost cells: the cell and face versions differ in where the low-side
   * pairs start (coarsen.cpp:38-41 vs coarsenBi_CT.cpp:38-41) and in the
   * clamp at the array edge (coarsen.cpp:55 vs coarsenBi_CT.cpp:54). */
  /* Left */
  for (int k = 0; k < nv; k++)
    for (int i = 0; i < ng / 2; i++)
      for (int j = 0; j < ng / 2; j++) {
        int i1 = nxminb - 2 * i - 1, j1 = nyminb - 2 * j - 1;
        Q[IX(o, dad, nv, k, nxminb - i, nyminb - j)] = SUM(son[0], k, i1, j1);
        j1 = nymaxb + 2 * j;
        Q[IX(o, dad, nv, k, nxminb - i, nymaxb + j)] = SUM(son[2], k, i1, j1);
      }
  for (int i = 0; i <= nxminb; i++)
    for (int j = nymin; j <= ny2; j++) {
      int j1 = 2 * j - nymin;
      int ny2j = j + ny2 - 1 - (ng - 2);
      int i1 = nxminb - 2 * i - 1;
      if (i1 < 0) i1 = 0;
      for (int k = 0; k < nv; k++) {
        Q[IX(o, dad, nv, k, nxminb - i, j)] = SUM(son[0], k, i1, j1);
        Q[IX(o, dad, nv, k, nxminb - i, ny2j)] = SUM(son[2], k, i1, j1);
      }
    }
  /* Right */
  for (int k = 0; k < nv; k++)
    for (int i = 0; i < ng / 2; i++)
      for (int j = 0; j < ng / 2; j++) {
        int i1 = nxmaxb + 2 * i, j1 = nyminb - 2 * j - 1;
        Q[IX(o, dad, nv, k, nxmaxb + i, nyminb - j)] = SUM(son[1], k, i1, j1);
        j1 = nymaxb + 2 * j;
        Q[IX(o, dad, nv, k, nxmaxb + i, nymaxb + j)] = SUM(son[3], k, i1, j1);
      }
  for (int i = 0; i < ng; i++)
    for (int j = nymin; j <= ny2; j++) {
      int j1 = 2 * j - nymin;
      int ny2j = j + ny2 - 1 - (ng - 2);
      int i1 = nxmaxb + 2 * i;
      if (i1 + 1 > nx - 1) i1 = nx - 2;
      for (int k = 0; k < nv; k++) {
        Q[IX(o, dad, nv, k, nxmaxb + i, j)] = SUM(son[1], k, i1, j1);
        Q[IX(o, dad, nv, k, nxmaxb + i, ny2j)] = SUM(son[3], k, i1, j1);
      }
    }
  /* Bottom */
  for (int k = 0; k < nv; k++)
    for (int j = 0; j < ng / 2; j++)
      for (int i = 0; i < ng / 2; i++) {
        int j1 = nyminb - 2 * j - 1, i1 = nxminb - 2 * i - 1;
        Q[IX(o, dad, nv, k, nxminb - i, nyminb - j)] = SUM(son[0], k, i1, j1);
        i1 = nxmaxb + 2 * i;
        Q[IX(o, dad, nv, k, nxmaxb + i, nyminb - j)] = SUM(son[1], k, i1, j1);
      }
  for (int i = nxmin; i <= nx2; i++)
    for (int j = 0; j <= nyminb; j++) {
      int i1 = 2 * i - nxmin;
      int nx2i = i + nx2 - 1 - (ng - 2);
      int j1 = nyminb - 2 * j - 1;
      if (j1 < 0) j1 = 0;
      for (int k = 0; k < nv; k++) {
        Q[IX(o, dad, nv, k, i, nyminb - j)] = SUM(son[0], k, i1, j1);
        Q[IX(o, dad, nv, k, nx2i, nyminb - j)] = SUM(son[1], k, i1, j1);
      }
    }
  /* Top */
  for (int k = 0; k < nv; k++)
    for (int j = 0; j < ng / 2; j++)
      for (int i = 0; i < ng / 2; i++) {
        int j1 = nymaxb + 2 * j, i1 = nxminb - 2 * i - 1;
        Q[IX(o, dad, nv, k, nxminb - i, nymaxb + j)] = SUM(son[2], k, i1, j1);
        i1 = nxmaxb + 2 * i;
        Q[IX(o, dad, nv, k, nxmaxb + i, nymaxb + j)] = SUM(son[3], k, i1, j1);
      }
  for (int i = nxmin; i <= nx2; i++)
    for (int j = 0; j < ng; j++) {
      int i1 = 2 * i - nxmin;
      int nx2i = i + nx2 - 1 - (ng - 2);
      int j1 = nymaxb + 2 * j;
      if (j1 + 1 > ny - 1) j1 = ny - 2;
      for (int k = 0; k < nv; k++) {
        Q[IX(o, dad, nv, k, i, nymaxb + j)] = SUM(son[2], k, i1, j1);
        Q[IX(o, dad, nv, k, nx2i, nymaxb + j)] = SUM(son[3], k, i1, j1);
      }
    }
#undef SUM
#undef I2
#undef J2
}

/* -------------------------------------------------- updatelpup/down.cpp */
/* updatelpup.cpp:4-118 */
static void updatelpup(oracle *o, int nb, const int *s) {
  int (*lp)[8] = o->lp;
  int nsr, nl2 = lp[nb][0] + 1;
  lp[s[0]][0] = nl2; lp[s[0]][1] = nb; lp[s[0]][3] = 0; lp[s[0]][5] = s[1]; lp[s[0]][7] = s[2];
  if (lp[nb][4] == -1 || o->leafs[lp[nb][4]]) lp[s[0]][4] = lp[nb][4];
  else { nsr = lp[lp[nb][4]][2] + 1; lp[s[0]][4] = nsr; lp[nsr][5] = s[0]; }
  if (lp[nb][6] == -1 || o->leafs[lp[nb][6]]) lp[s[0]][6] = lp[nb][6];
  else { nsr = lp[lp[nb][6]][2] + 2; lp[s[0]][6] = nsr; lp[nsr][7] = s[0]; }
  lp[s[1]][0] = nl2; lp[s[1]][1] = nb; lp[s[1]][3] = 1; lp[s[1]][4] = s[0]; lp[s[1]][7] = s[3];
  if (lp[nb][5] == -1 || o->leafs[lp[nb][5]]) lp[s[1]][5] = lp[nb][5];
  else { nsr = lp[lp[nb][5]][2]; lp[s[1]][5] = nsr; lp[nsr][4] = s[1]; }
  if (lp[nb][6] == -1 || o->leafs[lp[nb][6]]) lp[s[1]][6] = lp[nb][6];
  else { nsr = lp[lp[nb][6]][2] + 3; lp[s[1]][6] = nsr; lp[nsr][7] = s[1]; }
  lp[s[2]][0] = nl2; lp[s[2]][1] = nb; lp[s[2]][3] = 2; lp[s[2]][5] = s[3]; lp[s[2]][6] = s[0];
  if (lp[nb][4] == -1 || o->leafs[lp[nb][4]]) lp[s[2]][4] = lp[nb][4];
  else { nsr = lp[lp[nb][4]][2] + 3; lp[s[2]][4] = nsr; lp[nsr][5] = s[2]; }
  if (lp[nb][7] == -1 || o->leafs[lp[nb][7]]) lp[s[2]][7] = lp[nb][7];
  else { nsr = lp[lp[nb][7]][2]; lp[s[2]][7] = nsr; lp[nsr][6] = s[2]; }
  lp[s[3]][0] = nl2; lp[s[3]][1] = nb; lp[s[3]][3] = 3; lp[s[3]][4] = s[2]; lp[s[3]][6] = s[1];
  if (lp[nb][5] == -1 || o->leafs[lp[nb][5]]) lp[s[3]][5] = lp[nb][5];
  else { nsr = lp[lp[nb][5]][2] + 2; lp[s[3]][5] = nsr; lp[nsr][4] = s[3]; }
  if (lp[nb][7] == -1 || o->leafs[lp[nb][7]]) lp[s[3]][7] = lp[nb][7];
  else { nsr = lp[lp[nb][7]][2] + 1; lp[s[3]][7] = nsr; lp[nsr][6] = s[3]; }
  o->leafs[nb] = 0;
  for (int q = 0; q < 4; q++) o->leafs[s[q]] = 1;
  o->nbleafs += 4;
  o->iref[nb] = 0; o->icoarse[nb] = 0;
  for (int q = 0; q < 4; q++) o->icoarse[s[q]] = 0;
}

/* updatelpdown.cpp:4-54 */
static void updatelpdown(oracle *o, int dad, const int *s) {
  int (*lp)[8] = o->lp;
  o->leafs[dad] = 1;
  for (int q = 0; q < 4; q++) o->leafs[s[q]] = 0;
  o->nbleafs -= 3;
  int nb1 = lp[dad][4];
  if (nb1 != -1 && !o->leafs[nb1]) { nb1 = lp[lp[nb1][2]][5]; lp[nb1][5] = dad; lp[lp[nb1][7]][5] = dad; }
  nb1 = lp[dad][5];
  if (nb1 != -1 && !o->leafs[nb1]) { nb1 = lp[nb1][2]; lp[nb1][4] = dad; lp[lp[nb1][7]][4] = dad; }
  nb1 = lp[dad][6];
  if (nb1 != -1 && !o->leafs[nb1]) { nb1 = lp[lp[nb1][2]][7]; lp[nb1][7] = dad; lp[lp[nb1][5]][7] = dad; }
  nb1 = lp[dad][7];
  if (nb1 != -1 && !o->leafs[nb1]) { nb1 = lp[nb1][2]; lp[nb1][6] = dad; lp[lp[nb1][5]][6] = dad; }
}

/* --------------------------------------------------------------- admesh */
/* criteria.cpp:6-44 with max4diff (misc.cpp:13-20) */
static void criteria(oracle *o, int nb) {
  double grad = 0;
  const double rT = 0.05, cT = 1.0;
  static const int var[4] = {4, 0, 5, 6};
  for (int i = o->nxmin; i <= o->nxmax; i++)
    for (int j = o->nymin; j <= o->nymax; j++) {
      for (int q = 0; q < 4; q++) {
        int k = var[q];
        double c0 = Qc(o->W, nb, k, i, j);
        double dm = MMAX(EPS, fabs(c0));
        double d1 = fabs(Qc(o->W, nb, k, i + 1, j) - c0);
        double d2 = MMAX(d1, fabs(Qc(o->W, nb, k, i - 1, j) - c0));
        d1 = MMAX(d2, fabs(Qc(o->W, nb, k, i, j + 1) - c0));
        d2 = MMAX(d1, fabs(Qc(o->W, nb, k, i, j - 1) - c0));
        grad = MMAX(grad, d2 / dm);
      }
      if (grad >= rT) {
        if (o->lp[nb][0] < o->c.maxlevs - 1) { o->iref[nb] = 1; o->icoarse[nb] = 0; }
        return;
      }
    }
  if (grad <= cT) o->icoarse[nb] = 1;
}

/* admesh.cpp:17-102 with markref.cpp, critneighup.cpp, critneighdown.cpp;
 * with mref / mcrs non-NULL the caller's marks take criteria's place, set as
 * criteria.cpp:31-43 sets them (leaves only, no refinement on the finest
 * level, a refine mark cancelling a coarsen mark) */
static int admesh_with(oracle *o, const unsigned char *mref, const unsigned char *mcrs) {
  int (*lp)[8] = o->lp;
  int maxlevs = o->c.maxlevs;
  for (int nb = 0; nb < o->lastActive; nb++) { o->iref[nb] = 0; o->icoarse[nb] = 0; }
  for (int nb = 0; nb < o->lastActive; nb++) {
    if (!o->leafs[nb] || lp[nb][0] < 0) continue;
    if (!mref) {
      criteria(o, nb);
    } else if (mref[nb]) {
      if (lp[nb][0] < maxlevs - 1) o->iref[nb] = 1;
    } else if (mcrs[nb]) {
      o->icoarse[nb] = 1;
    }
  }
  for (int nl = maxlevs - 1; nl >= 0; nl--)        /* critneighup.cpp:6-34 */
    for (int nb = 0; nb < o->lastActive; nb++)
      if (o->iref[nb] && lp[nb][0] == nl)
        for (int d = 4; d < 8; d++) {
          int n1 = lp[nb][d];
          if (n1 != -1 && lp[n1][0] < lp[nb][0]) o->iref[n1] = 1;
        }
  for (int nl = 0; nl < maxlevs - 1; nl++)
    for (int nb = 0; nb < o->lastActive; nb++)
      if (lp[nb][0] == nl && o->iref[nb]) {
        int s[4];
        if (lp[nb][2] == 0) {
          s[0] = o->lastActive; s[1] = s[0] + 1; s[2] = s[0] + 2; s[3] = s[0] + 3;
          lp[nb][2] = s[0];
          o->lastActive += 4;
          if (o->lastActive - 1 >= o->maxblocks) return fail(o, "nblocks exceeded maxblocks");
        } else {
          s[0] = lp[nb][2]; s[1] = lp[s[0]][5]; s[2] = lp[s[0]][7]; s[3] = lp[s[2]][5];
        }
        if (refine(o, nb, s)) return -1;
        updatelpup(o, nb, s);
        if (refine_bi(o, nb, s)) return -1;
      }
  for (int nb = 0; nb < o->lastActive; nb++)       /* critneighdown.cpp:6-33 */
    if (o->icoarse[nb])
      for (int d = 4; d < 8; d++) {
        int n1 = lp[nb][d];
        if (n1 != -1 && !o->leafs[n1]) o->icoarse[nb] = 0;
      }
  for (int nl = maxlevs - 1; nl >= 1; nl--)
    for (int nb = 0; nb < o->lastActive; nb++)
      if (o->icoarse[nb] && lp[nb][3] == 0 && lp[nb][0] == nl) {
        int dad = lp[nb][1];
        int s[4] = {nb, lp[nb][5], lp[nb][7], 0};
        s[3] = lp[s[1]][7];
        if (o->icoarse[s[1]] && o->icoarse[s[2]] && o->icoarse[s[3]]) {
          coarsen_field(o, o->U, 8, 0, dad, s);
          if (cons2prim(o, o->U, dad, 0)) return -1;
          updatelpdown(o, dad, s);
          coarsen_field(o, o->Bi, 2, 1, dad, s);
        }
      }
  return 0;
}

static int admesh(oracle *o) { return admesh_with(o, NULL, NULL); }

/* ------------------------------------------------------------ IC2Dtype.cpp */
static void set_w(oracle *o, int nb, int i, int j, const double *w) {
  for (int k = 0; k < 8; k++) Qc(o->W, nb, k, i, j) = w[k];
}

/* IC2Dtype.cpp:6-190 for the reference ICs; extensions below */
static int ic2dtype(oracle *o, int nb) {
  double g, tEnd;
  double r4[4] = {0}, p4[4] = {0}, bx4[4] = {0}, by4[4] = {0};
  int ic = o->c.ic;
  switch (ic) {
    case OR_IC_SST: tEnd = 0.2; g = 2.0; { double p[4] = {0.1, 1.0, 1.0, 0.1}, r[4] = {0.125, 1.0, 1.0, 0.125}; memcpy(p4, p, 32); memcpy(r4, r, 32); } break;
    case OR_IC_SST1: tEnd = 0.2; g = 2.0; { double p[4] = {1.0, 0.1, 0.1, 1.0}, r[4] = {1.0, 0.125, 0.125, 1.0}; memcpy(p4, p, 32); memcpy(r4, r, 32); } break;
    case OR_IC_SSTY: tEnd = 0.2; g = 2.0; { double p[4] = {0.1, 0.1, 1.0, 1.0}, r[4] = {0.125, 0.125, 1.0, 1.0}; memcpy(p4, p, 32); memcpy(r4, r, 32); } break;
    case OR_IC_BWX: tEnd = 0.2; g = 2.0; { double p[4] = {0.1, 1.0, 1.0, 0.1}, r[4] = {0.125, 1.0, 1.0, 0.125}, bx[4] = {0.75, 0.75, 0.75, 0.75}, by[4] = {-1.0, 1.0, 1.0, -1.0}; memcpy(p4, p, 32); memcpy(r4, r, 32); memcpy(bx4, bx, 32); memcpy(by4, by, 32); } break;
    case OR_IC_BWX1: tEnd = 0.2; g = 2.0; { double p[4] = {1.0, 0.1, 0.1, 1.0}, r[4] = {1.0, 0.125, 0.125, 1.0}, bx[4] = {0.75, 0.75, 0.75, 0.75}, by[4] = {1.0, -1.0, -1.0, 1.0}; memcpy(p4, p, 32); memcpy(r4, r, 32); memcpy(bx4, bx, 32); memcpy(by4, by, 32); } break;
    case OR_IC_BWY: tEnd = 0.2; g = 2.0; { double p[4] = {0.1, 0.1, 1.0, 1.0}, r[4] = {0.125, 0.125, 1.0, 1.0}, by[4] = {0.75, 0.75, 0.75, 0.75}, bx[4] = {-1.0, -1.0, 1.0, 1.0}; memcpy(p4, p, 32); memcpy(r4, r, 32); memcpy(bx4, bx, 32); memcpy(by4, by, 32); } break;
    case OR_IC_BWY1: tEnd = 0.2; g = 2.0; { double p[4] = {1.0, 1.0, 0.1, 0.1}, r[4] = {1.0, 1.0, 0.125, 0.125}, by[4] = {0.75, 0.75, 0.75, 0.75}, bx[4] = {1.0, 1.0, -1.0, -1.0}; memcpy(p4, p, 32); memcpy(r4, r, 32); memcpy(bx4, bx, 32); memcpy(by4, by, 32); } break;
    case OR_IC_ROTOR: g = 1.4; tEnd = 0.295; break;
    case OR_IC_OT: g = 5.0 / 3.0; tEnd = 3.14159265358979323846; break;
    case OR_IC_BLAST: g = 1.4; tEnd = 0.1; break;
    case OR_IC_KH: g = 5.0 / 3.0; tEnd = 1.0; break;
    default: return fail(o, "no valid initial condition");
  }
  if (o->c.gamma_override > 0) g = o->c.gamma_override;
  if (o->c.tend_override > 0) tEnd = o->c.tend_override;
  o->gamma = g;
  o->tEnd = tEnd;
  int lev = o->lp[nb][0], ng = o->ng;
  double dxl = o->dx[lev], dyl = o->dy[lev];
  for (int i = 0; i < o->nx; i++) {
    double x = ((i + o->icoord[nb][0] - ng) + 0.5) * dxl - (o->c.geom_ref ? o->dx[0] : 0.0);
    for (int j = 0; j < o->ny; j++) {
      double y = ((j + o->icoord[nb][1] - ng) + 0.5) * dyl - (o->c.geom_ref ? o->dy[0] : 0.0);
      double w[8] = {0};
      if (ic == OR_IC_ROTOR) {      /* IC2Dtype.cpp:90-113 */
        double radius = sqrt((x - 0.5) * (x - 0.5) + (y - 0.5) * (y - 0.5));
        double fr = (23. - 200. * radius) / 3.;
        w[4] = 0.5;
        w[5] = 2.5 / (sqrt(4 * PI_REF));
        if (radius <= 0.1) { w[0] = 10.; w[1] = -(y - 0.5) / 0.1; w[2] = (x - 0.5) / 0.1; }
        else if (radius > 0.1 && radius < 0.115) {
          w[0] = (1 + 9. * fr); w[1] = (-(y - 0.5) * fr / 0.1); w[2] = (x - 0.5) * fr / 0.1;
        } else w[0] = 1.;
      } else if (ic == OR_IC_OT) {  /* extension: Orszag-Tang on [0,2pi]^2 */
        const double pi = 3.14159265358979323846, s4p = sqrt(4.0 * pi);
        w[0] = 25.0 / (36.0 * pi); w[4] = 5.0 / (12.0 * pi);
        w[1] = -sin(y); w[2] = sin(x);
        w[5] = -sin(y) / s4p; w[6] = sin(2.0 * x) / s4p;
      } else if (ic == OR_IC_BLAST) { /* extension: seeded blast, parameters drawn by the caller */
        const double *P = o->c.ic_param; /* r0, p_in, |B|, theta, xc, yc */
        double rr = sqrt((x - P[4]) * (x - P[4]) + (y - P[5]) * (y - P[5]));
        w[0] = 1.0; w[4] = rr < P[0] ? P[1] : 0.1;
        w[5] = P[2] * cos(P[3]); w[6] = P[2] * sin(P[3]);
      } else if (ic == OR_IC_KH) {  /* extension: seeded Kelvin-Helmholtz, a_k in ic_param */
        const double pi = 3.14159265358979323846;
        int in = fabs(y - 0.5) <= 0.25;
        w[0] = in ? 2.0 : 1.0; w[1] = in ? 0.5 : -0.5; w[4] = 2.5;
        w[5] = 0.1 / sqrt(4.0 * pi);
        double env = exp(-(y - 0.25) * (y - 0.25) / 0.01) + exp(-(y - 0.75) * (y - 0.75) / 0.01);
        double v = 0.0;
        for (int kk = 0; kk < 16; kk++) v += o->c.ic_param[kk] * sin(2.0 * pi * (kk + 1) * x);
        w[2] = v * env;
      } else {                      /* IC2Dtype.cpp:114-168 quadrants */
        int q;
        if (x >= 0.5 && y >= 0.5) q = 0;
        else if (x < 0.5 && y >= 0.5) q = 1;
        else if (x < 0.5 && y < 0.5) q = 2;
        else q = 3;
        w[0] = r4[q]; w[4] = p4[q]; w[5] = bx4[q]; w[6] = by4[q];
      }
      set_w(o, nb, i, j, w);
    }
  }
  /* IC2Dtype.cpp:172-189 face B from averages of the cell values */
  for (int i = 0; i < o->nx; i++)
    for (int j = 0; j < o->ny; j++) {
      if (i < o->nx - 1) Qf(o->Bi, nb, 0, i + 1, j) = 0.5 * (Qc(o->W, nb, 5, i, j) + Qc(o->W, nb, 5, i + 1, j));
      else Qf(o->Bi, nb, 0, 0, j) = Qf(o->Bi, nb, 0, 1, j);
      if (j < o->ny - 1) Qf(o->Bi, nb, 1, i, j + 1) = 0.5 * (Qc(o->W, nb, 6, i, j) + Qc(o->W, nb, 6, i, j + 1));
      else Qf(o->Bi, nb, 1, i, 0) = Qf(o->Bi, nb, 1, i, 1);
    }
  return 0;
}

/* ------------------------------------------------------------------ API */
oracle *oracle_create(const oracle_cfg *cfg) {
  oracle *o = (oracle *)calloc(1, sizeof(oracle));
  if (!o) return NULL;
  o->c = *cfg;
  if (o->c.nghosts <= 0) o->c.nghosts = 2;
  if (o->c.nroots_x <= 0) o->c.nroots_x = 2;
  if (o->c.nroots_y <= 0) o->c.nroots_y = 2;
  if (o->c.maxlevs <= 0 || o->c.maxlevs > MAXLEV) { free(o); return NULL; }
  o->ng = o->c.nghosts;
  o->nx = o->c.nx_int + 2 * o->ng;
  o->ny = o->c.ny_int + 2 * o->ng;
  o->nv = 8;
  /* parameters.cpp:10-21 */
  o->nxmin = o->ng; o->nxmax = o->nx - 1 - o->ng;
  o->nymin = o->ng; o->nymax = o->ny - 1 - o->ng;
  o->nxminb = o->nxmin - 1; o->nxmaxb = o->nxmax + 1;
  o->nyminb = o->nymin - 1; o->nymaxb = o->nymax + 1;
  o->nxp1 = o->nxmaxb; o->nyp1 = o->nymaxb;
  o->nx2 = (o->nx - 1) / 2; o->ny2 = (o->ny - 1) / 2;
  o->nroots = o->c.nroots_x * o->c.nroots_y;
  /* block IDs are never freed (admesh.cpp:33-51); a full tree bounds them */
  long long mb = 0, p = 1;
  for (int l = 0; l < o->c.maxlevs; l++) { mb += p; p *= 4; }
  o->maxblocks = (int)(mb * o->nroots);
  /* meshblock.cpp:90-96 */
  if (o->c.geom_ref) {
    o->dx[0] = o->c.lenx / ((double)o->c.nroots_x * (o->nx - 2 * o->ng - 1));
    o->dy[0] = o->c.leny / ((double)o->c.nroots_y * (o->ny - 2 * o->ng - 1));
  } else {
    o->dx[0] = o->c.lenx / ((double)o->c.nroots_x * (o->nx - 2 * o->ng));
    o->dy[0] = o->c.leny / ((double)o->c.nroots_y * (o->ny - 2 * o->ng));
  }
  for (int l = 1; l < MAXLEV; l++) { o->dx[l] = o->dx[l - 1] / 2.; o->dy[l] = o->dy[l - 1] / 2.; }
  size_t MB = (size_t)o->maxblocks;
  o->cell = (size_t)8 * o->nx * o->ny;
  o->face = (size_t)2 * o->nx * o->ny;
  o->lp = calloc(MB, sizeof(int[8]));
  o->icoord = calloc(MB, sizeof(int[2]));
  o->leafs = calloc(MB, 1); o->iref = calloc(MB, 1); o->icoarse = calloc(MB, 1);
  o->bflag = calloc(MB, 4);
  o->ib_cap = 4 * (int)MB + 4;
  o->ib = calloc((size_t)o->ib_cap, sizeof(int[3]));
  o->U = calloc(MB * o->cell, 8); o->Us = calloc(MB * o->cell, 8); o->W = calloc(MB * o->cell, 8);
  o->ff = calloc(MB * o->cell, 8); o->gg = calloc(MB * o->cell, 8);
  o->Bi = calloc(MB * o->face, 8); o->Bis = calloc(MB * o->face, 8);
  o->EMF = calloc(MB * (size_t)o->nx * o->ny, 8);
  o->nthreads = o->c.nthreads;
#ifdef _OPENMP
  if (o->nthreads <= 0) o->nthreads = omp_get_max_threads();
#else
  o->nthreads = 1;
#endif
  o->scratch = calloc((size_t)o->nthreads * 6 * o->cell, 8);
  if (!o->lp || !o->U || !o->Us || !o->W || !o->ff || !o->gg || !o->Bi || !o->Bis || !o->EMF ||
      !o->scratch || !o->ib || !o->bflag) {
    oracle_destroy(o);
    return NULL;
  }
  return o;
}

void oracle_destroy(oracle *o) {
  if (!o) return;
  free(o->lp); free(o->icoord); free(o->leafs); free(o->iref); free(o->icoarse); free(o->bflag);
  free(o->ib); free(o->U); free(o->Us); free(o->W); free(o->ff); free(o->gg); free(o->Bi);
  free(o->Bis); free(o->EMF); free(o->scratch);
  free(o);
}

/* basegrid.cpp:4-89 (2 x 2 roots) generalised to N_x x N_y, row-major IDs */
int oracle_init(oracle *o) {
  int nrx = o->c.nroots_x, nry = o->c.nroots_y;
  int ni = o->nx - 2 * o->ng, nj = o->ny - 2 * o->ng;
  for (int jr = 0; jr < nry; jr++)
    for (int ir = 0; ir < nrx; ir++) {
      int nb = jr * nrx + ir;
      int *l = o->lp[nb];
      l[0] = 0; l[1] = 0; l[2] = 0; l[3] = 0;
      int per = o->c.periodic;
      l[4] = ir > 0 ? nb - 1 : (per ? nb + nrx - 1 : -1);
      l[5] = ir < nrx - 1 ? nb + 1 : (per ? nb - (nrx - 1) : -1);
      l[6] = jr > 0 ? nb - nrx : (per ? nb + nrx * (nry - 1) : -1);
      l[7] = jr < nry - 1 ? nb + nrx : (per ? nb - nrx * (nry - 1) : -1);
      o->icoord[nb][0] = ir * ni;
      o->icoord[nb][1] = jr * nj;
      o->leafs[nb] = 1;
      o->iref[nb] = 1;
    }
  o->lastActive = o->nroots;
  o->nbleafs = o->nroots;
  for (int nb = 0; nb < o->lastActive; nb++) {
    if (ic2dtype(o, nb)) return -1;
    prim2cons(o, nb);
  }
  /* main.cpp:99-101 W2U again, then the initial remesh (main.cpp:110) */
  for (int nb = 0; nb < o->lastActive; nb++) if (o->leafs[nb]) prim2cons(o, nb);
  o->dt = 0.0;   /* dom.dt is read before its first assignment in the reference */
  o->dtn = 0.0;
  if (o->c.dt_fixed > 0) o->dt = o->dtn = o->c.dt_fixed;
  o->t = 0.0;
  o->count = 0;
  if (o->c.maxlevs > 1 && admesh(o)) return -1;
  o->initialised = 1;
  return 0;
}

int oracle_done(const oracle *o) { return !(o->t <= o->tEnd); }

/* main.cpp:128-247 */
int oracle_step(oracle *o) {
  if (!o->initialised) return fail(o, "oracle_init not called");
  if (o->err_set) return -1;
  int *leaf = (int *)malloc(sizeof(int) * (o->lastActive + 1));
  int nL = 0;
  locate_bounds(o);
  for (int nb = 0; nb < o->lastActive; nb++) if (o->leafs[nb]) leaf[nL++] = nb;
  fill_cc(o, o->U);
  fill_fc(o, o->Bi, 2);
  int bad = 0;
#pragma omp parallel for schedule(dynamic, 1) num_threads(o->nthreads) reduction(| : bad)
  for (int l = 0; l < nL; l++) bad |= muscl_rk(o, leaf[l], 1) != 0;
  if (bad) { free(leaf); return -1; }
  fill_fc(o, o->Bi, 2);
  fill_fc(o, o->ff, 8);
  fill_fc(o, o->gg, 8);
  if (ct2d(o, o->Us, o->Bi, 1, o->Bis)) { free(leaf); return -1; }
  fill_cc(o, o->Us);
#pragma omp parallel for schedule(dynamic, 1) num_threads(o->nthreads) reduction(| : bad)
  for (int l = 0; l < nL; l++) bad |= muscl_rk(o, leaf[l], 2) != 0;
  if (bad) { free(leaf); return -1; }
  if (o->c.diffusion) {
#pragma omp parallel for schedule(dynamic, 1) num_threads(o->nthreads)
    for (int l = 0; l < nL; l++)
      if (o->lp[leaf[l]][0] >= o->c.maxlevs - 2) diffuse(o, o->U, leaf[l]);
  }
  fill_fc(o, o->ff, 8);
  fill_fc(o, o->gg, 8);
  if (ct2d(o, o->U, o->Bis, 2, o->Bi)) { free(leaf); return -1; }
  fill_cc(o, o->U);
  /* main.cpp:209-230 dt; note lambda1 takes |rho| + c_f,x (W[..][0], main.cpp:222) */
  double lambda = 1.E6;
  double *lam_b = (double *)malloc(sizeof(double) * (nL + 1));
#pragma omp parallel for schedule(dynamic, 1) num_threads(o->nthreads) reduction(| : bad)
  for (int l = 0; l < nL; l++) {
    int nb = leaf[l];
    if (cons2prim(o, o->U, nb, 0)) { bad |= 1; continue; }
    double l1 = 0., l2 = 0.;
    for (int i = o->nxmin; i <= o->nxmax; i++)
      for (int j = o->nymin; j <= o->nymax; j++) {
        double w[8], a, ca, can, cf;
        for (int k = 0; k < 8; k++) w[k] = Qc(o->W, nb, k, i, j);
        wavespeeds(w, o->gamma, 5, &a, &ca, &can, &cf);
        l1 = SMAX(l1, fabs(w[0]) + cf);
        wavespeeds(w, o->gamma, 6, &a, &ca, &can, &cf);
        l2 = SMAX(l2, fabs(w[1]) + cf);
      }
    l1 = SMAX(l1, l2);
    lam_b[l] = SMIN(o->dx[o->lp[nb][0]], o->dy[o->lp[nb][0]]) / l1;
  }
  if (bad) { free(leaf); free(lam_b); return -1; }
  for (int l = 0; l < nL; l++) lambda = SMIN(lambda, lam_b[l]);
  free(lam_b);
  free(leaf);
  o->count = o->count + 1;
  if (o->c.dt_fixed > 0) {
    o->t = o->t + o->c.dt_fixed;
  } else {
    o->t = o->t + o->dtn;
    o->dt = o->dtn;
    o->dtn = o->c.cfl * lambda;
    if (o->dtn < 0 || isnan(o->dtn)) return fail(o, "invalid dt");
  }
  if (o->c.maxlevs > 1 && !o->no_remesh && admesh(o)) return -1;
  return 0;
}

int oracle_run(oracle *o, int nsteps, double t_stop) {
  while (o->t <= o->tEnd) {
    if (nsteps >= 0 && o->count >= nsteps) break;
    if (t_stop >= 0 && o->t > t_stop) break;
    if (oracle_step(o)) return -1;
  }
  return 0;
}

void oracle_info(const oracle *o, int *ints, double *dbls) {
  ints[0] = o->lastActive; ints[1] = o->nbleafs; ints[2] = o->count; ints[3] = o->nx;
  ints[4] = o->ny; ints[5] = o->maxblocks; ints[6] = o->ng; ints[7] = o->err_set;
  dbls[0] = o->t; dbls[1] = o->dt; dbls[2] = o->dtn; dbls[3] = o->gamma; dbls[4] = o->tEnd;
  dbls[5] = o->dx[0]; dbls[6] = o->dy[0]; dbls[7] = 0;
}

int64_t oracle_get(const oracle *o, int what, void *dst) {
  size_t nA = (size_t)o->lastActive;
  size_t n;
  const void *src;
  size_t esz = 8;
  switch (what) {
    case OR_GET_U: src = o->U; n = nA * o->cell; break;
    case OR_GET_US: src = o->Us; n = nA * o->cell; break;
    case OR_GET_W: src = o->W; n = nA * o->cell; break;
    case OR_GET_FF: src = o->ff; n = nA * o->cell; break;
    case OR_GET_GG: src = o->gg; n = nA * o->cell; break;
    case OR_GET_BI: src = o->Bi; n = nA * o->face; break;
    case OR_GET_BIS: src = o->Bis; n = nA * o->face; break;
    case OR_GET_EMF: src = o->EMF; n = nA * o->nx * o->ny; break;
    case OR_GET_LP: src = o->lp; n = nA * 8; esz = 4; break;
    case OR_GET_ICOORD: src = o->icoord; n = nA * 2; esz = 4; break;
    case OR_GET_LEAFS: src = o->leafs; n = nA; esz = 1; break;
    default: return -1;
  }
  if (dst) memcpy(dst, src, n * esz);
  return (int64_t)n;
}

int oracle_set(oracle *o, int what, const double *src) {
  size_t nA = (size_t)o->lastActive;
  if (what == OR_GET_U) memcpy(o->U, src, nA * o->cell * 8);
  else if (what == OR_GET_BI) memcpy(o->Bi, src, nA * o->face * 8);
  else return -1;
  return 0;
}

const char *oracle_error(const oracle *o) { return o->err_set ? o->err : ""; }

/* the sequential ghost fill of the current tree applied to an external array
 * [lastActive][nv][ny][nx]; kind 0 = cell (boundary.cpp), 1 = face
 * (boundaryfc.cpp), 2 = edge (boundaryec.cpp) */
void oracle_set_remesh(oracle *o, int on) { o->no_remesh = !on; }
int oracle_admesh(oracle *o) { return admesh(o); }
int oracle_admesh_marked(oracle *o, const unsigned char *iref, const unsigned char *icoarse) {
  if (!iref || !icoarse) return fail(o, "null marks");
  return admesh_with(o, iref, icoarse);
}

int oracle_fill(oracle *o, double *field, int nv, int kind) {
  locate_bounds(o);
  fld f = {field, nv, kind};
  ghostfill(o, &f);
  return 0;
}
