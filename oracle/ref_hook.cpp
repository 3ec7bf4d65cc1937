// Test infrastructure, not product code.
//
// Hook object linked with the UNMODIFIED reference sources (main.cpp and the
// numerical files of spaceauk/AMR2D_MHD) by oracle/ref.mk.  The recipe compiles
// main.cpp with `-Dadmesh=amr_ref_admesh_hook -Dsave4py=amr_ref_save4py`, so
// main's own calls land here:
//
//   * main.cpp:110 (initial remesh) and main.cpp:246 (remesh at the end of
//     every step) call amr_ref_admesh_hook, which dumps the full-precision
//     state (U, W, face B, quadtree) AFTER delegating to the real admesh().
//     The dump taken at the end of step n is therefore the state after the
//     two RK stages, CT, the dt reduction and the remesh of step n, i.e. the
//     state the time loop starts step n+1 from.
//   * main.cpp:242,262 call amr_ref_save4py, a no-op: the reference's text
//     writer (savedata.cpp) keeps only 6 significant digits.
//
// The hook also pins one undefined behaviour of the reference: main.cpp reads
// dom.dt (an uninitialised member, defs.hpp:90) in the RK stages of the first
// step before main.cpp:231 assigns it.  The first call (the initial remesh,
// main.cpp:110) sets dom.dt = 0, which is what the reference sees in practice
// on a fresh stack and what every other implementation here assumes.
//
// Environment:
//   AMR_REF_DUMP   path prefix; dumps go to <prefix>_<step>.bin
//   AMR_REF_EVERY  dump every k-th step (default 1) and the last step of the
//                  time loop; step 0 = after the initial remesh, before it
//   AMR_REF_STOP   exit(0) right after the dump of this step (default: run on)
//   AMR_REF_TLOG   path of a log that receives, for EVERY step (dumped or
//                  not), one record: i32 step, i32 lastActive, i32 leaves,
//                  i32 0, f64 t, f64 dt (the dump header's t and dt)
#include "defs.hpp"

#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <cstdint>

void admesh(meshblock &dom);

namespace {

int g_calls = 0;      // number of hook calls so far
double g_t = 0.0;     // replica of main's t (t = t + dt, main.cpp:231)

long env_long(const char *name, long dflt) {
  const char *v = std::getenv(name);
  if (!v || !*v) return dflt;
  return std::strtol(v, nullptr, 10);
}

void put_i32(FILE *f, int32_t v) { std::fwrite(&v, 4, 1, f); }
void put_f64(FILE *f, double v) { std::fwrite(&v, 8, 1, f); }

// Layout of a dump (little endian):
//   "AMRREF01" | i32 nx ny nvar maxlevs nghosts lastActive nbleafs step |
//   f64 t dt gamma dx0 dy0 |
//   per block nb < lastActive: i32 lp[8], i32 icoord[2], i32 leaf |
//   f64 U[lastActive][nvar][ny][nx] | f64 W[...same...] |
//   f64 Bi[lastActive][2][ny][nx]
void dump(meshblock &dom, int step) {
  const char *prefix = std::getenv("AMR_REF_DUMP");
  if (!prefix || !*prefix) return;
  char path[4096];
  std::snprintf(path, sizeof(path), "%s_%d.bin", prefix, step);
  FILE *f = std::fopen(path, "wb");
  if (!f) { std::perror(path); std::exit(3); }
  std::fwrite("AMRREF01", 1, 8, f);
  put_i32(f, dom.nx); put_i32(f, dom.ny); put_i32(f, dom.nvar);
  put_i32(f, maxlevs); put_i32(f, nghosts);
  put_i32(f, dom.lastActive); put_i32(f, dom.nbleafs); put_i32(f, step);
  put_f64(f, g_t); put_f64(f, (double)dom.dt); put_f64(f, (double)dom.gamma);
  put_f64(f, (double)dom.dx[0]); put_f64(f, (double)dom.dy[0]);
  for (int nb = 0; nb < dom.lastActive; nb++) {
    for (int q = 0; q < 8; q++) put_i32(f, dom.lp[nb][q]);
    put_i32(f, dom.icoord[nb][0]); put_i32(f, dom.icoord[nb][1]);
    put_i32(f, dom.leafs[nb] ? 1 : 0);
  }
  for (int pass = 0; pass < 2; pass++) {
    real ****Q = pass == 0 ? dom.U : dom.W;
    for (int nb = 0; nb < dom.lastActive; nb++)
      for (int k = 0; k < dom.nvar; k++)
        for (int j = 0; j < dom.ny; j++)
          for (int i = 0; i < dom.nx; i++) put_f64(f, (double)Q[i][j][k][nb]);
  }
  for (int nb = 0; nb < dom.lastActive; nb++)
    for (int k = 0; k < 2; k++)
      for (int j = 0; j < dom.ny; j++)
        for (int i = 0; i < dom.nx; i++) put_f64(f, dom.Bi[i][j][k][nb]);
  std::fclose(f);
}

FILE *g_tlog = nullptr;

void log_step(meshblock &dom, int step) {
  const char *path = std::getenv("AMR_REF_TLOG");
  if (!path || !*path) return;
  if (!g_tlog) {
    g_tlog = std::fopen(path, "wb");
    if (!g_tlog) { std::perror(path); std::exit(3); }
  }
  int32_t leaves = 0;
  for (int nb = 0; nb < dom.lastActive; nb++) leaves += dom.leafs[nb] ? 1 : 0;
  put_i32(g_tlog, step); put_i32(g_tlog, dom.lastActive); put_i32(g_tlog, leaves); put_i32(g_tlog, 0);
  put_f64(g_tlog, g_t); put_f64(g_tlog, (double)dom.dt);
  std::fflush(g_tlog);
}

}  // namespace

void amr_ref_admesh_hook(meshblock &dom) {
  int step;
  if (g_calls == 0) {
    dom.dt = 0;  // see the header comment
    step = 0;
  } else {
    g_t = g_t + dom.dt;
    step = g_calls;
  }
  g_calls++;
  admesh(dom);
  log_step(dom, step);
  long every = env_long("AMR_REF_EVERY", 1);
  long stop = env_long("AMR_REF_STOP", -1);
  // the time loop ends after this step when t > tEnd (main.cpp:128): that
  // step is dumped whatever `every` says
  const bool last = !(g_t <= (double)dom.tEnd);
  if (every > 0 && (step % every == 0 || last)) dump(dom, step);
  if (stop >= 0 && step >= stop) {
    if (every <= 0 || step % every != 0) dump(dom, step);
    std::fflush(stdout);
    std::exit(0);
  }
}

void amr_ref_save4py(meshblock &, int, real) {}

// Declared (never called) by several reference files; savedata.cpp, which
// defines it, is not linked.
void savearray(meshblock &, real ***, string) {}
