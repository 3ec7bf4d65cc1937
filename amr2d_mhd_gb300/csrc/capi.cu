// extern "C" boundary (include/amr2d_mhd.h).  No C++ exception crosses it.
#include <cstdio>
#include <cstring>
#include <exception>
#include <fstream>
#include <new>
#include <string>

#include "engine.hpp"

struct amr_handle {
  amr::Engine engine;
};

namespace {
// Every entry point but amr_step_end first finishes a step that
// amr_step_begin left in flight, so each sees the state after that step.
template <typename F>
int guarded(amr_handle *h, F &&f, bool finish_pending = true) {
  if (!h) return AMR_E_ARG;
  try {
    if (finish_pending && h->engine.step_pending())
      if (int rc = h->engine.step_end()) return rc;
    return f(h->engine);
  } catch (const std::bad_alloc &) {
    h->engine.last_error = "host out of memory";
    return AMR_E_OOM;
  } catch (const std::exception &e) {
    h->engine.last_error = e.what();
    return AMR_E_STATE;
  }
}
void copy_name(char *dst, const std::string &s) {
  std::memset(dst, 0, 16);
  std::strncpy(dst, s.c_str(), 15);
}
}  // namespace

extern "C" {

int amr_abi_version(void) { return AMR_ABI_VERSION; }

const char *amr_status_string(int s) {
  switch (s) {
    case AMR_OK: return "ok";
    case AMR_E_CONFIG: return "invalid configuration";
    case AMR_E_CUDA: return "CUDA error";
    case AMR_E_OOM: return "out of memory";
    case AMR_E_MAXBLOCKS: return "block budget exceeded";
    case AMR_E_PRESSURE: return "zero or negative pressure";
    case AMR_E_NAN: return "NaN encountered";
    case AMR_E_DT: return "invalid dt";
    case AMR_E_HLLC: return "HLLC wave-speed trap";
    case AMR_E_STATE: return "call out of order";
    case AMR_E_TIMEOUT: return "device wait timed out";
    case AMR_E_UNSUPPORTED: return "unsupported option";
    case AMR_E_ARG: return "bad argument";
    case AMR_E_TOO_LARGE: return "size above a fixed scratch capacity";
    case AMR_E_CT: return "incorrect psi produced (upwind CT EMF)";
    default: return "unknown status";
  }
}

// defaults = the reference's shipped input.txt and defs.hpp constants
void amr_config_default(amr_config *c) {
  if (!c) return;
  std::memset(c, 0, sizeof(*c));
  c->struct_size = sizeof(amr_config);
  c->nx = 16; c->ny = 16; c->nvar = 8;
  c->lenx = 1.0; c->leny = 1.0;
  c->cfl = 0.5;
  copy_name(c->ic, "rotor");
  copy_name(c->limiter, "MC");
  copy_name(c->flux, "RUSA");
  c->maxlevs = 5;
  c->nghosts = 2;
  c->nroots_x = 2; c->nroots_y = 2;
  c->periodic = 0;
  c->geometry = 0;
  c->gamma = 0.0;
  c->t_end = 0.0;
  c->precision = AMR_FP64;
}

// main.cpp:43-64
int amr_config_from_input(const char *path, amr_config *c) {
  if (!path || !c) return AMR_E_ARG;
  std::ifstream f(path);
  if (!f.is_open()) return AMR_E_CONFIG;  // "Unable to open the file..."
  int nx, ny, nvar;
  double lx, ly, cfl;
  std::string ic, lim, flux;
  if (!(f >> nx >> ny >> nvar >> lx >> ly >> cfl >> ic >> lim >> flux)) return AMR_E_CONFIG;
  c->nx = nx; c->ny = ny; c->nvar = nvar;
  c->lenx = lx; c->leny = ly; c->cfl = cfl;
  if (ic.size() > 15 || lim.size() > 15 || flux.size() > 15) return AMR_E_CONFIG;
  copy_name(c->ic, ic);
  copy_name(c->limiter, lim);
  copy_name(c->flux, flux);
  return AMR_OK;
}

int amr_config_blast(uint64_t seed, int32_t index, amr_config *c) {
  if (!c || index < 0) return AMR_E_ARG;
  amr_config_default(c);
  copy_name(c->ic, "blast");
  copy_name(c->limiter, "MC");
  copy_name(c->flux, "HLLE");
  c->cfl = 0.2;
  c->geometry = 1;
  c->gamma = 1.4;
  c->t_end = 0.1;
  int maxlevs = 3;
  amr::blast_draw(seed, index, c->ic_param, maxlevs);
  c->maxlevs = maxlevs;
  return AMR_OK;
}

int amr_config_kh(uint64_t seed, amr_config *c) {
  if (!c) return AMR_E_ARG;
  amr_config_default(c);
  copy_name(c->ic, "KH");
  copy_name(c->limiter, "MC");
  copy_name(c->flux, "RUSA");
  c->maxlevs = 1;
  c->nroots_x = 16;
  c->nroots_y = 16;
  c->periodic = 1;
  c->geometry = 1;
  c->gamma = 5.0 / 3.0;
  c->dt_fixed = 2e-4;
  c->t_end = 1.0;
  amr::kh_draw(seed, c->ic_param);
  return AMR_OK;
}

int amr_create_batch(const amr_config *cfgs, int32_t n, amr_handle **out) {
  if (!cfgs || !out || n <= 0) return AMR_E_ARG;
  *out = nullptr;
  for (int q = 0; q < n; q++)
    if (cfgs[q].struct_size != static_cast<int32_t>(sizeof(amr_config))) return AMR_E_CONFIG;
  amr_handle *h = new (std::nothrow) amr_handle();
  if (!h) return AMR_E_OOM;
  int rc = guarded(h, [&](amr::Engine &e) { return e.create(cfgs, n); });
  if (rc != AMR_OK) {
    std::fprintf(stderr, "amr_create: %s\n", h->engine.last_error.c_str());
    delete h;
    return rc;
  }
  *out = h;
  return AMR_OK;
}

int amr_create(const amr_config *cfg, amr_handle **out) { return amr_create_batch(cfg, 1, out); }

int amr_destroy(amr_handle *h) {
  delete h;
  return AMR_OK;
}

int amr_set_stream(amr_handle *h, void *s) {
  return guarded(h, [&](amr::Engine &e) { return e.set_stream(static_cast<cudaStream_t>(s)); });
}

int amr_last_error(const amr_handle *h, char *buf, size_t len) {
  if (!h || !buf || len == 0) return AMR_E_ARG;
  std::strncpy(buf, h->engine.last_error.c_str(), len - 1);
  buf[len - 1] = 0;
  return AMR_OK;
}

int amr_init(amr_handle *h) { return guarded(h, [](amr::Engine &e) { return e.init(); }); }
int amr_step(amr_handle *h) { return guarded(h, [](amr::Engine &e) { return e.step(); }); }
int amr_step_begin(amr_handle *h) { return guarded(h, [](amr::Engine &e) { return e.step_begin(); }); }
int amr_step_end(amr_handle *h) { return guarded(h, [](amr::Engine &e) { return e.step_end(); }, false); }
int amr_run(amr_handle *h, int64_t n) { return guarded(h, [&](amr::Engine &e) { return e.run(n); }); }
int amr_get_info(amr_handle *h, int32_t q, amr_info *o) {
  return guarded(h, [&](amr::Engine &e) { return e.info(q, o); });
}
int amr_locate_bounds(amr_handle *h) { return guarded(h, [](amr::Engine &e) { return e.api_locate_bounds(); }); }
int amr_boundary(amr_handle *h, int32_t f) { return guarded(h, [&](amr::Engine &e) { return e.api_boundary(f); }); }
int amr_muscl2d_rk(amr_handle *h, int32_t s) { return guarded(h, [&](amr::Engine &e) { return e.api_muscl2d_rk(s); }); }
int amr_ct2d(amr_handle *h, int32_t s) { return guarded(h, [&](amr::Engine &e) { return e.api_ct2d(s); }); }
int amr_cfl_dt(amr_handle *h, double *l) { return guarded(h, [&](amr::Engine &e) { return e.api_cfl_dt(l); }); }
int amr_admesh(amr_handle *h) { return guarded(h, [](amr::Engine &e) { return e.api_admesh(); }); }
int amr_set_tree(amr_handle *h, int32_t q, int32_t na, int32_t nbl, const int32_t *lp, const int32_t *ic,
                 const uint8_t *lf, double t, double dt, double dtn, int64_t steps) {
  return guarded(h, [&](amr::Engine &e) { return e.api_set_tree(q, na, nbl, lp, ic, lf, t, dt, dtn, steps); });
}
int amr_get_tree(amr_handle *h, int32_t q, int32_t *lp, int32_t *ic, uint8_t *lf, int32_t cap) {
  return guarded(h, [&](amr::Engine &e) { return e.get_tree(q, lp, ic, lf, cap); });
}
int amr_download(amr_handle *h, int32_t q, int32_t f, double *d, int64_t n) {
  return guarded(h, [&](amr::Engine &e) { return e.download(q, f, d, n); });
}
int amr_upload(amr_handle *h, int32_t q, int32_t f, const double *s, int64_t n) {
  return guarded(h, [&](amr::Engine &e) { return e.upload(q, f, s, n); });
}

int amr_set_remesh(amr_handle *h, int32_t on) {
  return guarded(h, [&](amr::Engine &e) { return e.set_remesh(on != 0); });
}
int amr_profile_enable(amr_handle *h, int32_t on) {
  return guarded(h, [&](amr::Engine &e) { return e.profile_enable(on != 0); });
}
int amr_profile_read(amr_handle *h, amr_profile *o) {
  return guarded(h, [&](amr::Engine &e) { return e.profile_read(o); });
}

int amr_admesh_marked(amr_handle *h, const uint8_t *iref, const uint8_t *icoarse, int32_t n) {
  return guarded(h, [&](amr::Engine &e) { return e.api_admesh_marked(iref, icoarse, n); });
}
int amr_criteria_flags(amr_handle *h, uint8_t *iref, uint8_t *icoarse, int32_t cap) {
  return guarded(h, [&](amr::Engine &e) { return e.api_criteria_flags(iref, icoarse, cap); });
}
int amr_criteria(amr_handle *h, double *grad, int32_t cap) {
  return guarded(h, [&](amr::Engine &e) { return e.api_criteria(grad, cap); });
}

int amr_autotune(amr_handle *h, int32_t reps, char *report, size_t len) {
  return guarded(h, [&](amr::Engine &e) { return e.autotune(reps, report, len); });
}

int amr_save4py(amr_handle *h, int32_t inst, int32_t id, const char *dir, int32_t digits, char *name_out,
                size_t name_len) {
  return guarded(h, [&](amr::Engine &e) { return e.save4py(inst, id, dir, digits, name_out, name_len); });
}
int amr_checkpoint_save(amr_handle *h, const char *path) {
  return guarded(h, [&](amr::Engine &e) { return e.checkpoint_save(path); });
}
int amr_checkpoint_load(amr_handle *h, const char *path) {
  return guarded(h, [&](amr::Engine &e) { return e.checkpoint_load(path); });
}

int amr_adjoint_enable(amr_handle *h, int32_t on) {
  return guarded(h, [&](amr::Engine &e) { return e.adjoint_enable(on != 0); });
}
int amr_adjoint_seed(amr_handle *h, int32_t inst, int32_t field, const double *lam, int64_t count) {
  return guarded(h, [&](amr::Engine &e) { return e.adjoint_seed(inst, field, lam, count); });
}
int amr_adjoint_step(amr_handle *h) { return guarded(h, [](amr::Engine &e) { return e.adjoint_step(); }); }
int amr_adjoint_read(amr_handle *h, int32_t inst, int32_t field, double *lam, int64_t count) {
  return guarded(h, [&](amr::Engine &e) { return e.adjoint_read(inst, field, lam, count); });
}
int amr_adjoint_recorded(amr_handle *h, int32_t *steps) {
  if (!steps) return AMR_E_ARG;
  return guarded(h, [&](amr::Engine &e) {
    *steps = e.adjoint_recorded();
    return AMR_OK;
  });
}

}  // extern "C"
