// Test infrastructure, not product code.
//
// Known-answer harness linked with the reference's own riemannS.o, misc.o and
// slopelimiter.o (oracle/ref.mk target `kat`).  Reads cases from a binary file
// and writes the reference's answers:
//   riemann case:  i32 flux (0 RUSA 1 HLLE 2 HLLC 3 HLLD 4 ROE), i32 dir (0 x, 1 y),
//                  f64 gamma, f64 wL[8], f64 wR[8]  ->  i32 status, f64 flux[8]
//   limiter case:  i32 limiter (index into kLim), f64 r, f64 eta  ->  f64 phi
// Usage: kat.x riemann|limiter <in> <out>
#include "defs.hpp"

#include <cstdio>
#include <cstring>
#include <exception>
#include <string>
#include <vector>

void riemannS(string fluxMth, vector<real> wL, vector<real> wR, real gamma, char direc, vector<real> &flux);
real slopelimiter(string limiter, real r, real eta);

int main(int argc, char **argv) {
  if (argc != 4) return 2;
  FILE *in = std::fopen(argv[2], "rb");
  FILE *out = std::fopen(argv[3], "wb");
  if (!in || !out) return 3;
  static const char *kFlux[] = {"RUSA", "HLLE", "HLLC", "HLLD", "ROE"};
  static const char *kLim[] = {"1st", "noSL", "minmod", "VanLeer", "Superbee", "MC", "Koren", "Cada3rd"};
  if (!std::strcmp(argv[1], "riemann")) {
    int32_t fl, dir;
    double g, w[16];
    while (std::fread(&fl, 4, 1, in) == 1 && std::fread(&dir, 4, 1, in) == 1 &&
           std::fread(&g, 8, 1, in) == 1 && std::fread(w, 8, 16, in) == 16) {
      vector<real> wL(w, w + 8), wR(w + 8, w + 16), f(8, 0.0);
      int32_t st = 0;
      try {
        riemannS(kFlux[fl], wL, wR, g, dir ? 'y' : 'x', f);
      } catch (const std::exception &) {
        st = 1;
      }
      std::fwrite(&st, 4, 1, out);
      std::fwrite(f.data(), 8, 8, out);
    }
  } else {
    int32_t li;
    double r, eta;
    while (std::fread(&li, 4, 1, in) == 1 && std::fread(&r, 8, 1, in) == 1 && std::fread(&eta, 8, 1, in) == 1) {
      double phi = slopelimiter(kLim[li], r, eta);
      std::fwrite(&phi, 8, 1, out);
    }
  }
  std::fclose(in);
  std::fclose(out);
  return 0;
}
