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

bool ic_prepare(IcId ic, const double *P, const IcBlock &b, double gamma, IcDev &d, double *tab) {
  const int n = b.n;
  std::memset(&d, 0, sizeof d);
  d.ic = ic;
  d.icoord_x = b.icoord_x;
  d.icoord_y = b.icoord_y;
  d.dx = b.dx;
  d.dy = b.dy;
  d.shift_x = b.shift_x;
  d.shift_y = b.shift_y;
  d.gamma = gamma;
  d.tab = -1;
  Quad q;
  if (quad_states(ic, q)) {  // IC2Dtype.cpp:20-68
    for (int k = 0; k < 4; k++) {
      d.c[k] = q.r[k];
      d.c[4 + k] = q.p[k];
      d.c[8 + k] = q.bx[k];
      d.c[12 + k] = q.by[k];
    }
    return false;
  }
  // the cell centres, as the kernel forms them
  auto X = [&](int i) { return ((i + b.icoord_x - b.ng) + 0.5) * b.dx - b.shift_x; };
  auto Y = [&](int j) { return ((j + b.icoord_y - b.ng) + 0.5) * b.dy - b.shift_y; };
  switch (ic) {
    case IC_ROTOR:  // IC2Dtype.cpp:80
      d.c[0] = 2.5 / (std::sqrt(4 * kPiRef));
      return false;
    case IC_OT:  // Orszag-Tang on [0, 2 pi]^2
      d.c[0] = 25.0 / (36.0 * kPi);
      d.c[1] = 5.0 / (12.0 * kPi);
      d.c[2] = std::sqrt(4.0 * kPi);
      for (int i = 0; i < n; i++) {
        tab[i] = std::sin(X(i));
        tab[n + i] = std::sin(2.0 * X(i));
        tab[2 * n + i] = std::sin(Y(i));
      }
      return true;
    case IC_BLAST:  // P: r0, p_in, |B|, theta, xc, yc
      d.c[0] = P[0];
      d.c[1] = P[1];
      d.c[2] = P[2] * std::cos(P[3]);
      d.c[3] = P[2] * std::sin(P[3]);
      d.c[4] = P[4];
      d.c[5] = P[5];
      return false;
    case IC_KH:  // P: a_1..a_16
      d.c[0] = 0.1 / std::sqrt(4.0 * kPi);
      for (int i = 0; i < n; i++) {
        const double x = X(i), y = Y(i);
        double v = 0.0;
        for (int k = 0; k < 16; k++) v += P[k] * std::sin(2.0 * kPi * (k + 1) * x);
        tab[i] = v;
        tab[n + i] = std::exp(-(y - 0.25) * (y - 0.25) / 0.01) + std::exp(-(y - 0.75) * (y - 0.75) / 0.01);
        tab[2 * n + i] = 0.0;
      }
      return true;
    default:
      return false;
  }
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
