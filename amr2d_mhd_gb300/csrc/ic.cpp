// Initial conditions and the host-side helpers of amr_init.
#include "ic.hpp"

#include <cmath>
#include <cstring>

namespace amr {

namespace {
constexpr double kPiRef = 3.14159265359;  // defs.hpp:23
constexpr double kPi = 3.14159265358979323846;

struct Quad { double r[4], p[4], bx[4], by[4]; };

// IC2Dtype.cpp:20-68: the four quadrant states, index 0 = (x>=0.5, y>=0.5),
// 1 = (x<0.5, y>=0.5), 2 = (x<0.5, y<0.5), 3 = (x>=0.5, y<0.5)
bool quad_states(IcId ic, Quad &q) {
  std::memset(&q, 0, sizeof q);
  auto set = [](double *d, double a, double b, double c, double e) { d[0] = a; d[1] = b; d[2] = c; d[3] = e; };
  switch (ic) {
    case IC_SST: set(q.p, 0.1, 1.0, 1.0, 0.1); set(q.r, 0.125, 1.0, 1.0, 0.125); return true;
    case IC_SST1: set(q.p, 1.0, 0.1, 0.1, 1.0); set(q.r, 1.0, 0.125, 0.125, 1.0); return true;
    case IC_SSTY: set(q.p, 0.1, 0.1, 1.0, 1.0); set(q.r, 0.125, 0.125, 1.0, 1.0); return true;
    case IC_BWX:
      set(q.p, 0.1, 1.0, 1.0, 0.1); set(q.r, 0.125, 1.0, 1.0, 0.125);
      set(q.bx, 0.75, 0.75, 0.75, 0.75); set(q.by, -1.0, 1.0, 1.0, -1.0); return true;
    case IC_BWX1:
      set(q.p, 1.0, 0.1, 0.1, 1.0); set(q.r, 1.0, 0.125, 0.125, 1.0);
      set(q.bx, 0.75, 0.75, 0.75, 0.75); set(q.by, 1.0, -1.0, -1.0, 1.0); return true;
    case IC_BWY:
      set(q.p, 0.1, 0.1, 1.0, 1.0); set(q.r, 0.125, 0.125, 1.0, 1.0);
      set(q.by, 0.75, 0.75, 0.75, 0.75); set(q.bx, -1.0, -1.0, 1.0, 1.0); return true;
    case IC_BWY1:
      set(q.p, 1.0, 1.0, 0.1, 0.1); set(q.r, 1.0, 1.0, 0.125, 0.125);
      set(q.by, 0.75, 0.75, 0.75, 0.75); set(q.bx, 1.0, 1.0, -1.0, -1.0); return true;
    default: return false;
  }
}
}  // namespace

IcId ic_from_name(const std::string &s) {
  static const char *names[] = {"SST", "SST1", "SSTy", "BWx", "BWx1", "BWy", "BWy1", "rotor",
                                "OT", "blast", "KH"};
  for (int i = 0; i < IC_INVALID; i++)
    if (s == names[i]) return static_cast<IcId>(i);
  return IC_INVALID;
}

void ic_params(IcId ic, double &gamma, double &tend) {
  switch (ic) {
    case IC_ROTOR: gamma = 1.4; tend = 0.295; break;  // IC2Dtype.cpp:77-78
    case IC_OT: gamma = 5.0 / 3.0; tend = kPi; break;
    case IC_BLAST: gamma = 1.4; tend = 0.1; break;
    case IC_KH: gamma = 5.0 / 3.0; tend = 1.0; break;
    default: gamma = 2.0; tend = 0.2; break;          // SST*/BW* (IC2Dtype.cpp:22-67)
  }
}

void ic_fill(IcId ic, const double *P, const IcBlock &b, double *W, double *Bi) {
  const int n = b.n, nn = n * n;
  Quad q;
  const bool quad = quad_states(ic, q);
  for (int i = 0; i < n; i++) {
    const double x = ((i + b.icoord_x - b.ng) + 0.5) * b.dx - b.shift_x;
    for (int j = 0; j < n; j++) {
      const double y = ((j + b.icoord_y - b.ng) + 0.5) * b.dy - b.shift_y;
      double w[8] = {0, 0, 0, 0, 0, 0, 0, 0};
      if (quad) {
        int k;
        if (x >= 0.5 && y >= 0.5) k = 0;
        else if (x < 0.5 && y >= 0.5) k = 1;
        else if (x < 0.5 && y < 0.5) k = 2;
        else k = 3;
        w[0] = q.r[k]; w[4] = q.p[k]; w[5] = q.bx[k]; w[6] = q.by[k];
      } else if (ic == IC_ROTOR) {  // IC2Dtype.cpp:90-113
        const double radius = std::sqrt((x - 0.5) * (x - 0.5) + (y - 0.5) * (y - 0.5));
        const double fr = (23. - 200. * radius) / 3.;
        w[4] = 0.5;
        w[5] = 2.5 / (std::sqrt(4 * kPiRef));
        if (radius <= 0.1) {
          w[0] = 10.; w[1] = -(y - 0.5) / 0.1; w[2] = (x - 0.5) / 0.1;
        } else if (radius > 0.1 && radius < 0.115) {
          w[0] = (1 + 9. * fr); w[1] = (-(y - 0.5) * fr / 0.1); w[2] = (x - 0.5) * fr / 0.1;
        } else {
          w[0] = 1.;
        }
      } else if (ic == IC_OT) {  // Orszag-Tang on [0, 2 pi]^2
        const double s4p = std::sqrt(4.0 * kPi);
        w[0] = 25.0 / (36.0 * kPi); w[4] = 5.0 / (12.0 * kPi);
        w[1] = -std::sin(y); w[2] = std::sin(x);
        w[5] = -std::sin(y) / s4p; w[6] = std::sin(2.0 * x) / s4p;
      } else if (ic == IC_BLAST) {  // P: r0, p_in, |B|, theta, xc, yc
        const double rr = std::sqrt((x - P[4]) * (x - P[4]) + (y - P[5]) * (y - P[5]));
        w[0] = 1.0; w[4] = rr < P[0] ? P[1] : 0.1;
        w[5] = P[2] * std::cos(P[3]); w[6] = P[2] * std::sin(P[3]);
      } else if (ic == IC_KH) {  // P: a_1..a_16
        const bool in = std::fabs(y - 0.5) <= 0.25;
        w[0] = in ? 2.0 : 1.0; w[1] = in ? 0.5 : -0.5; w[4] = 2.5;
        w[5] = 0.1 / std::sqrt(4.0 * kPi);
        const double env = std::exp(-(y - 0.25) * (y - 0.25) / 0.01) +
                           std::exp(-(y - 0.75) * (y - 0.75) / 0.01);
        double v = 0.0;
        for (int k = 0; k < 16; k++) v += P[k] * std::sin(2.0 * kPi * (k + 1) * x);
        w[2] = v * env;
      }
      for (int k = 0; k < 8; k++) W[k * nn + j * n + i] = w[k];
    }
  }
  // IC2Dtype.cpp:172-189
  double *Bx = Bi, *By = Bi + nn;
  for (int i = 0; i < n; i++)
    for (int j = 0; j < n; j++) {
      if (i < n - 1) Bx[j * n + i + 1] = 0.5 * (W[5 * nn + j * n + i] + W[5 * nn + j * n + i + 1]);
      else Bx[j * n + 0] = Bx[j * n + 1];
      if (j < n - 1) By[(j + 1) * n + i] = 0.5 * (W[6 * nn + j * n + i] + W[6 * nn + (j + 1) * n + i]);
      else By[0 * n + i] = By[1 * n + i];
    }
}

void prim_to_cons(const double *W, double *U, int nn, double g) {
  for (int c = 0; c < nn; c++) {
    double w[8];
    for (int k = 0; k < 8; k++) w[k] = W[k * nn + c];
    U[0 * nn + c] = w[0];
    U[1 * nn + c] = w[1] * w[0];
    U[2 * nn + c] = w[2] * w[0];
    U[3 * nn + c] = w[3] * w[0];
    const double e = (w[4] / (g - 1)) + 0.5 * w[0] * (w[1] * w[1] + w[2] * w[2] + w[3] * w[3]);
    U[4 * nn + c] = e + 0.5 * (w[5] * w[5] + w[6] * w[6] + w[7] * w[7]);
    U[5 * nn + c] = w[5];
    U[6 * nn + c] = w[6];
    U[7 * nn + c] = w[7];
  }
}

double criteria_grad(const double *W, int n, int ng) {
  const int nn = n * n;
  static const int var[4] = {4, 0, 5, 6};
  double grad = 0;
  for (int i = ng; i <= n - 1 - ng; i++)
    for (int j = ng; j <= n - 1 - ng; j++)
      for (int q = 0; q < 4; q++) {
        const double *w = W + var[q] * nn;
        const double c0 = w[j * n + i];
        const double dm = 1.0E-15 > std::fabs(c0) ? 1.0E-15 : std::fabs(c0);
        double d = std::fabs(w[j * n + i + 1] - c0);
        double e = std::fabs(w[j * n + i - 1] - c0);
        d = d > e ? d : e;
        e = std::fabs(w[(j + 1) * n + i] - c0);
        d = d > e ? d : e;
        e = std::fabs(w[(j - 1) * n + i] - c0);
        d = d > e ? d : e;
        const double r = d / dm;
        grad = grad > r ? grad : r;
      }
  return grad;
}

}  // namespace amr

// ------------------------------------------------------------- seeded problems
namespace amr {

// MT19937-64 (Matsumoto & Nishimura; Nishimura 2000), written out so the draw
// does not depend on the standard library's distributions.
SeededDraw::SeededDraw(unsigned long long seed) {
  mt_[0] = seed;
  for (int i = 1; i < 312; i++)
    mt_[i] = 6364136223846793005ULL * (mt_[i - 1] ^ (mt_[i - 1] >> 62)) + static_cast<unsigned long long>(i);
  idx_ = 312;
}

unsigned long long SeededDraw::raw() {
  constexpr unsigned long long kUpper = 0xFFFFFFFF80000000ULL, kLower = 0x7FFFFFFFULL;
  constexpr unsigned long long kMatrix = 0xB5026F5AA96619E9ULL;
  if (idx_ >= 312) {
    for (int i = 0; i < 312; i++) {
      const unsigned long long x = (mt_[i] & kUpper) | (mt_[(i + 1) % 312] & kLower);
      unsigned long long xa = x >> 1;
      if (x & 1ULL) xa ^= kMatrix;
      mt_[i] = mt_[(i + 156) % 312] ^ xa;
    }
    idx_ = 0;
  }
  unsigned long long y = mt_[idx_++];
  y ^= (y >> 29) & 0x5555555555555555ULL;
  y ^= (y << 17) & 0x71D67FFFEDA60000ULL;
  y ^= (y << 37) & 0xFFF7EEE000000000ULL;
  y ^= y >> 43;
  return y;
}

double SeededDraw::uniform() { return static_cast<double>(raw() >> 11) * (1.0 / 9007199254740992.0); }

double SeededDraw::normal() {
  if (have_spare_) { have_spare_ = false; return spare_; }
  double u1 = uniform();
  const double u2 = uniform();
  if (u1 <= 0.0) u1 = 1.0 / 9007199254740992.0;
  const double r = std::sqrt(-2.0 * std::log(u1));
  spare_ = r * std::sin(2.0 * kPi * u2);
  have_spare_ = true;
  return r * std::cos(2.0 * kPi * u2);
}

void blast_draw(unsigned long long seed, int index, double P[6], int &maxlevs) {
  SeededDraw g(seed + static_cast<unsigned long long>(index));
  const double s4p = std::sqrt(4.0 * kPi);
  P[0] = 0.05 + 0.10 * g.uniform();
  P[1] = 5.0 + 45.0 * g.uniform();
  P[2] = (0.5 + 1.5 * g.uniform()) / s4p;
  P[3] = 0.5 * kPi * g.uniform();
  P[4] = 0.5;
  P[5] = 0.5;
  maxlevs = 3 + static_cast<int>(g.raw() >> 62);
}

void kh_draw(unsigned long long seed, double a[16]) {
  SeededDraw g(seed);
  for (int k = 0; k < 16; k++) a[k] = 1e-3 * g.normal();
}

}  // namespace amr
