// amr2d_mhd: the reference program's main() (main.cpp) on the GB300 library.
//
// Reads input.txt (main.cpp:43-64) and the same answers on standard input:
// first 2 = run a simulation, 1 = plot existing data (main.cpp:73-95; the
// plotting script is not part of this library, so 1 only says so), then,
// after the run, the variable to plot (main.cpp:264-277, read and ignored).
// Runs the time loop `while (t <= tEnd)` through the C ABI, prints one line
// per step as main.cpp:232 does, and writes <data>/<IC><id>t_<t>.dat
// (savedata.cpp) every 20 steps, between the dt reduction and admesh as
// main.cpp:240-246 does, and once more at the end (main.cpp:262).
// The reference's compile-time constants (defs.hpp:27-35: nghosts, maxlevs,
// CTtype, diffusion) are command-line options here.
#include <chrono>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <filesystem>
#include <iostream>
#include <string>

#include "amr2d_mhd.h"

namespace {

void usage() {
  std::printf(
      "usage: amr2d_mhd [--input FILE] [--data DIR] [--maxlevs N] [--nghosts N] [--ct-type 1|2]\n"
      "                 [--diffusion] [--precision fp64|fp32] [--save-every N] [--digits N] [--quiet]\n"
      "Reads FILE (default input.txt) and, on standard input, 2 (run) or 1 (plot existing data).\n"
      "Defaults: maxlevs 5, nghosts 2 (4 for WENO5), ct-type 1, fp64, a save every 20 steps into data/.\n");
}

int report(amr_handle *h, int rc, const char *what) {
  if (rc == AMR_OK) return 0;
  char msg[512] = {0};
  if (h) amr_last_error(h, msg, sizeof msg);
  std::fprintf(stderr, "%s: %s (%s)\n", what, amr_status_string(rc), msg);
  return rc;
}

bool int_arg(int argc, char **argv, int &i, int &out) {
  if (i + 1 >= argc) return false;
  char *end = nullptr;
  const long v = std::strtol(argv[++i], &end, 10);
  if (!end || *end) return false;
  out = static_cast<int>(v);
  return true;
}

}  // namespace

int main(int argc, char **argv) {
  std::string input = "input.txt", data = "data", precision = "fp64";
  int maxlevs = 5, nghosts = 0, ct_type = 1, diffusion = 0, every = 20, digits = 0;
  bool quiet = false;
  for (int i = 1; i < argc; i++) {
    const std::string a = argv[i];
    bool ok = true;
    if (a == "--help" || a == "-h") {
      usage();
      return 0;
    } else if (a == "--input" && i + 1 < argc) {
      input = argv[++i];
    } else if (a == "--data" && i + 1 < argc) {
      data = argv[++i];
    } else if (a == "--precision" && i + 1 < argc) {
      precision = argv[++i];
      ok = precision == "fp64" || precision == "fp32";
    } else if (a == "--maxlevs") {
      ok = int_arg(argc, argv, i, maxlevs);
    } else if (a == "--nghosts") {
      ok = int_arg(argc, argv, i, nghosts);
    } else if (a == "--ct-type") {
      ok = int_arg(argc, argv, i, ct_type);
    } else if (a == "--save-every") {
      ok = int_arg(argc, argv, i, every);
    } else if (a == "--digits") {
      ok = int_arg(argc, argv, i, digits);
    } else if (a == "--diffusion") {
      diffusion = 1;
    } else if (a == "--quiet") {
      quiet = true;
    } else {
      ok = false;
    }
    if (!ok) {
      std::fprintf(stderr, "bad argument: %s\n", a.c_str());
      usage();
      return 2;
    }
  }

  amr_config cfg;
  amr_config_default(&cfg);
  if (amr_config_from_input(input.c_str(), &cfg) != AMR_OK) {  // main.cpp:66-70
    std::printf("Unable to open the file...\n***Terminating program***\n");
    return 1;
  }
  cfg.maxlevs = maxlevs;
  cfg.nghosts = nghosts > 0 ? nghosts : (std::strcmp(cfg.limiter, "WENO5") == 0 ? 4 : 2);
  cfg.ct_type = ct_type;
  cfg.diffusion = diffusion;
  cfg.precision = precision == "fp32" ? AMR_FP32 : AMR_FP64;
  std::printf("Domain size is %d x %d with nvar=%d\nCFL=%g\n-----MHD solver-----\n", cfg.nx, cfg.ny, cfg.nvar,
              cfg.cfl);
  std::printf("Problems chosen: %s\nLimiter selected: %s\nTypes of Riemann Solver chosen: %s\n", cfg.ic,
              cfg.limiter, cfg.flux);

  std::printf("For plotting, (1) Use existing data (2) Run simulation and obtain new data\n");
  int choice = 2;
  if (!(std::cin >> choice)) choice = 2;
  if (choice == 1) {
    std::printf("Plotting existing data is left to the reference's call_plot.py; nothing to run.\n");
    return 0;
  }
  if (choice != 2) {
    std::printf("Error as wrong selection!\n");
    return 1;
  }

  amr_handle *h = nullptr;
  if (int rc = amr_create(&cfg, &h)) return report(h, rc, "amr_create");
  int rc = amr_init(h);
  if (!rc) rc = amr_set_remesh(h, 0);  // the save comes between the dt reduction and admesh
  if (rc) {
    report(h, rc, "amr_init");
    amr_destroy(h);
    return 1;
  }
  std::error_code ec;
  std::filesystem::create_directories(data, ec);
  if (ec) {
    std::fprintf(stderr, "cannot create %s: %s\n", data.c_str(), ec.message().c_str());
    amr_destroy(h);
    return 1;
  }

  std::printf("Entering main loop...\n");
  const auto t0 = std::chrono::steady_clock::now();
  amr_info inf;
  int simu = 0;
  char name[1024];
  for (;;) {
    if ((rc = amr_get_info(h, 0, &inf))) break;
    if (!(inf.t <= inf.t_end)) break;  // main.cpp:128
    if ((rc = amr_step(h))) break;
    if ((rc = amr_get_info(h, 0, &inf))) break;
    if (!quiet)  // main.cpp:232
      std::printf("%lld) At t=%g, dt=%g and # of blocks are %d\n", static_cast<long long>(inf.steps - 1), inf.t,
                  inf.dt, inf.last_active);
    if (every > 0 && inf.steps % every == 0) {  // main.cpp:240-243
      simu += 1;
      if ((rc = amr_save4py(h, 0, simu, data.c_str(), digits, name, sizeof name))) break;
    }
    if (cfg.maxlevs > 1 && (rc = amr_admesh(h))) break;  // main.cpp:246
  }
  if (rc) {
    report(h, rc, "time loop");
    amr_destroy(h);
    return 1;
  }
  const double wall = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  if ((rc = amr_save4py(h, 0, simu + 1, data.c_str(), digits, name, sizeof name))) {  // main.cpp:262
    report(h, rc, "save4py");
    amr_destroy(h);
    return 1;
  }
  std::printf("Finished at t=%g after %lld steps: %.3f s, %.3e cell-updates/s; last output %s\n", inf.t,
              static_cast<long long>(inf.steps), wall,
              wall > 0 ? static_cast<double>(inf.cell_updates) / wall : 0.0, name);
  std::string plot_var;
  std::cin >> plot_var;  // main.cpp:275, for the reference's plotting script
  amr_destroy(h);
  return 0;
}
