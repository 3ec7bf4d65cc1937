/*
 * amr2d_mhd.h — C ABI of the GB300 (sm_103a) per-block finite-volume update
 * of a 2-D block-structured AMR ideal-MHD solver (drop-in for the hot path of
 * spaceauk/AMR2D_MHD).
 *
 * The reference has no library API: its seam is the set of free functions
 * main() calls on a `meshblock&` (main.cpp:128-247).  Each entry point below
 * names the reference function it replaces.  Conventions:
 *   - plain C types only; an opaque handle owns one or more AMR problems
 *     ("instances"); all cell- and face-centred data stay resident on one GPU;
 *   - every call returns an amr_status (0 = ok, < 0 = error); the reference
 *     prints and throws on the same conditions, here the message is kept for
 *     amr_last_error();
 *   - one host thread per handle; work is issued on the handle's CUDA stream
 *     (amr_set_stream) and calls that return host data synchronise it.
 */
#ifndef AMR2D_MHD_H
#define AMR2D_MHD_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define AMR_ABI_VERSION 1

typedef enum amr_status {
  AMR_OK = 0,
  AMR_E_CONFIG = -1,      /* invalid option (the reference throws, e.g. slopelimiter.cpp:50) */
  AMR_E_CUDA = -2,        /* CUDA runtime error or no device */
  AMR_E_OOM = -3,         /* device allocation failed */
  AMR_E_MAXBLOCKS = -4,   /* admesh.cpp:42-45 "nblocks exceeded max limit" */
  AMR_E_PRESSURE = -5,    /* meshblock.cpp:136-142 / 164-170 zero or negative pressure */
  AMR_E_NAN = -6,         /* celledges.cpp:17-21, MUSCL2D.cpp:79-85, meshblock.cpp:171-176 */
  AMR_E_DT = -7,          /* main.cpp:235-238 invalid dt */
  AMR_E_HLLC = -8,        /* riemannS.cpp:269-276 */
  AMR_E_STATE = -9,       /* call out of order (e.g. amr_step before amr_init) */
  AMR_E_TIMEOUT = -10,    /* a bounded device wait gave up */
  AMR_E_UNSUPPORTED = -11,/* ROE with a magnetic field (riemannS.cpp:39-40), block size != 16 */
  AMR_E_ARG = -12,        /* bad pointer, size or index */
  AMR_E_TOO_LARGE = -13,  /* more blocks than a fixed-size scratch array holds */
  AMR_E_CT = -14          /* CT2D.cpp:68 "Incorrect psi produced" (ct_type 2) */
} amr_status;

typedef enum amr_precision {
  AMR_FP64 = 0,           /* plain path: identical arithmetic to the reference */
  AMR_FP32 = 1            /* FP32 bulk; FP64 pressure recovery, face B, dt and sums */
} amr_precision;

typedef enum amr_field {
  AMR_FIELD_U = 0,        /* conserved state U [blocks][8][ny+2g][nx+2g] */
  AMR_FIELD_US = 1,       /* RK stage state Us */
  AMR_FIELD_BI = 2,       /* face magnetic field Bi [blocks][2][..][..] (Bx at i-1/2, By at j-1/2) */
  AMR_FIELD_BIS = 3,      /* RK stage face field Bis */
  AMR_FIELD_FF = 4,       /* x fluxes ff (face i-1/2) */
  AMR_FIELD_GG = 5,       /* y fluxes gg (face j-1/2) */
  AMR_FIELD_EMF = 6,      /* corner EMF [blocks][1][..][..] */
  AMR_FIELD_W = 7         /* primitive state, computed from U on download */
} amr_field;

/* One AMR problem.  The first block of fields is input.txt (main.cpp:43-64);
 * the second block holds the reference's compile-time constants (defs.hpp)
 * and the extensions, each defaulting to the reference's value. */
typedef struct amr_config {
  int32_t struct_size;    /* sizeof(amr_config) */
  int32_t nx, ny, nvar;   /* interior cells per block and variables: 16 16 8 */
  double lenx, leny;      /* domain lengths: 1.0 1.0 */
  double cfl;             /* CFL number */
  char ic[16];            /* SST SST1 SSTy BWx BWx1 BWy BWy1 rotor | OT blast KH (extensions) */
  char limiter[16];       /* 1st noSL WENO2D minmod VanLeer Superbee MC Koren Cada3rd WENO3 WENO5 */
  char flux[16];          /* RUSA HLLE HLLC HLLD ROE */
  int32_t maxlevs;        /* refinement levels (defs.hpp:28, default 5) */
  int32_t nghosts;        /* ghost layers (defs.hpp:27, 2; 4 for WENO5) */
  int32_t nroots_x;       /* root blocks along x (2: defs.hpp:29 nbroots = 4) */
  int32_t nroots_y;
  int32_t periodic;       /* extension: periodic box instead of mirror outflow */
  int32_t geometry;       /* 0 = reference (dx0 = L/(sqrt(nroots)(nx-1)), shifted), 1 = L/cells */
  double gamma;           /* <= 0: the IC's own value (IC2Dtype.cpp) */
  double t_end;           /* <= 0: the IC's own value */
  double ic_param[24];    /* extension ICs (blast: r0, p_in, |B|, theta, xc, yc; KH: a_1..a_16) */
  int32_t precision;      /* amr_precision */
  int32_t reserved0;
  double dt_fixed;        /* extension: > 0 = every step uses this dt (no CFL
                             reduction, no lag); 0 = main.cpp:209-234 */
  int32_t ct_type;        /* defs.hpp:34 CTtype: 0 or 1 = basic EMF average, 2 = the
                             upwind-switched EMF of CT2D.cpp:28-75 */
  int32_t diffusion;      /* defs.hpp:35 diffusion: 1 = diffusivity.cpp after stage 2
                             on blocks at level >= maxlevs - 2 (main.cpp:190-193) */
  int32_t reserved[2];
} amr_config;

typedef struct amr_info {
  double t;               /* simulated time (main.cpp:231) */
  double dt;              /* dt used by the last step (dom.dt) */
  double dt_next;         /* dt the next-but-one step will use (main.cpp:234) */
  double t_end;
  double gamma;
  int64_t steps;          /* completed steps (main.cpp:233 count) */
  int32_t last_active;    /* block IDs in use (dom.lastActive) */
  int32_t n_leaves;       /* leaf blocks (count of dom.leafs) */
  int32_t nb_leafs;       /* the reference's own counter dom.nbleafs (updatelpup.cpp:109) */
  int32_t done;           /* 1 once t > t_end (main.cpp:128) */
  int32_t n_instances;
  int32_t nx_tot, ny_tot; /* block size with ghosts */
  int64_t cell_updates;   /* sum over completed steps of leaf interior cells */
} amr_info;

typedef struct amr_handle amr_handle;

/* ---- configuration ----------------------------------------------------- */
/* Defaults = the reference's constants; then parse an input.txt
 * (main.cpp:43-64: "nx ny nvar / lenx leny / CFL / IC limiter fluxMth"). */
void amr_config_default(amr_config *cfg);
int amr_config_from_input(const char *path, amr_config *cfg);
/* Seeded extension problems (no counterpart in the reference, which has
 * neither IC).  amr_config_blast: cylindrical blast instance `index` of the
 * batch `seed` (MT19937-64 seeded with seed + index; r0 ~ U[0.05,0.15],
 * p_in ~ U[5,50], |B| ~ U[0.5,2]/sqrt(4 pi), theta ~ U[0,pi/2], maxlevs ~
 * U{3..6}; gamma 1.4, MUSCL-MC + HLLE, CFL 0.2, outflow, 2 x 2 roots,
 * t_end 0.1).  amr_config_kh: frozen 256^2 periodic Kelvin-Helmholtz layer
 * (16 x 16 roots, maxlevs 1, MC + RUSA, gamma 5/3, dt_fixed 2e-4,
 * a_1..a_16 ~ N(0, (1e-3)^2) from MT19937-64 seeded with `seed`). */
int amr_config_blast(uint64_t seed, int32_t index, amr_config *cfg);
int amr_config_kh(uint64_t seed, amr_config *cfg);
int amr_abi_version(void);
const char *amr_status_string(int status);

/* ---- lifetime ------------------------------------------------------------ */
/* replaces meshblock::setSize / setType (meshblock.cpp:6-116) */
int amr_create(const amr_config *cfg, amr_handle **out);
/* several independent problems swept together; each keeps its own tree,
 * dt and end time */
int amr_create_batch(const amr_config *cfgs, int32_t n, amr_handle **out);
int amr_destroy(amr_handle *h);
int amr_set_stream(amr_handle *h, void *cuda_stream);
int amr_last_error(const amr_handle *h, char *buf, size_t len);

/* ---- the time loop --------------------------------------------------------- */
/* basegrid + IC2Dtype + W2U + initial admesh (main.cpp:97-116) */
int amr_init(amr_handle *h);
/* one iteration of main.cpp:128-247: ghost fills, two MUSCL2D + RK stages
 * with CT2D, the CFL dt reduction and admesh.  Instances that are done are
 * skipped. */
int amr_step(amr_handle *h);
/* amr_step in two halves (extension; the reference's loop has no such split):
 * amr_step_begin launches the step's device work on the handle's stream and
 * returns; amr_step_end waits for it and does the host half (t and dt, the
 * remesh, the ghost programs of the new trees).  Between the two the caller's
 * thread is free, e.g. for the host half of another handle's step on another
 * stream.  Any other call on the handle ends a step in flight first. */
int amr_step_begin(amr_handle *h);
int amr_step_end(amr_handle *h);
/* step until every instance is done, or `max_steps` steps (< 0: no limit) */
int amr_run(amr_handle *h, int64_t max_steps);
int amr_get_info(amr_handle *h, int32_t instance, amr_info *info);

/* ---- reference-function entry points (single instance) -------------------- */
int amr_locate_bounds(amr_handle *h);                        /* locate_bounds.cpp:35 */
int amr_boundary(amr_handle *h, int32_t field);              /* boundary/boundaryfc/boundaryec */
int amr_muscl2d_rk(amr_handle *h, int32_t step);             /* MUSCL2D + main.cpp:144-159 / 176-195 */
int amr_ct2d(amr_handle *h, int32_t step);                   /* CT2D.cpp:11 with its ghost fills */
/* main.cpp:209-230: the reference's `lambda` = dt / CFL of the current state */
int amr_cfl_dt(amr_handle *h, double *dt_per_cfl);
int amr_admesh(amr_handle *h);
/* on = 0: amr_step ends after the dt reduction (main.cpp:209-238) without the
 * closing admesh (main.cpp:246), so that the caller can act in between, as
 * main.cpp:240-243 saves the state there, and then call amr_admesh, which
 * remeshes on the same criterion the step would have used.  on = 1 (the
 * default) restores the closing admesh.  amr_init's initial admesh is not
 * affected. */
int amr_set_remesh(amr_handle *h, int32_t on);
/* criteria.cpp:6-44 on the current state of instance 0: grad[b] = the
 * largest relative jump of p, rho, Bx, By over the interior of leaf block b
 * (admesh refines where it is >= 0.05), -1 for blocks that are not leaves;
 * cap >= amr_info.last_active */
int amr_criteria(amr_handle *h, double *grad, int32_t cap);                               /* admesh.cpp:17 */
/* criteria.cpp's flags (:31, :43) of instance 0: iref[b] = 1 where a leaf's
 * criterion is >= 0.05 below the finest level, icoarse[b] = 1 where it is
 * below 0.05; 0 elsewhere and for non-leaves (admesh then applies the
 * neighbour rule of critneighup.cpp); cap >= amr_info.last_active */
int amr_criteria_flags(amr_handle *h, uint8_t *iref, uint8_t *icoarse, int32_t cap);
/* admesh.cpp:17-102 on instance 0 with the caller's marks in place of
 * criteria.cpp's (the prolongation / restriction of chosen blocks): for each
 * leaf b, iref[b] != 0 refines it (dropped on the finest level), else
 * icoarse[b] != 0 marks it for coarsening; entries of non-leaves are
 * ignored.  The neighbour rules (critneighup.cpp, critneighdown.cpp), the
 * four-sibling rule and the refine / coarsen operators (refine.cpp,
 * refineBi_CT.cpp, coarsen.cpp, coarsenBi_CT.cpp) are admesh's, so marks
 * equal to amr_criteria_flags give amr_admesh's result.  n >= last_active. */
int amr_admesh_marked(amr_handle *h, const uint8_t *iref, const uint8_t *icoarse, int32_t n);

/* riemannS (riemannS.cpp:7-56) on the GPU for n independent face states:
 * wL, wR and flux_out are [n][8] arrays in host memory (primitive states
 * rho u v w p Bx By Bz; fluxes of the conserved variables).  flux: 0 RUSA,
 * 1 HLLE, 2 HLLC, 3 HLLD, 4 ROE (riemannS.cpp:297-395); dir_y: 0 x face, 1
 * y face (the reference's rotation); mag_field: the reference's
 * compile-time MAG_field (defs.hpp:32), 1 in every run of the time loop, 0
 * its hydrodynamic configuration (no field rotation; the only one in which
 * ROE is accepted, riemannS.cpp:39-40: with mag_field = 1 ROE returns
 * AMR_E_UNSUPPORTED).  status (may be NULL) receives 0 or AMR_E_HLLC (the
 * traps of riemannS.cpp:269-276) per pair.  FP64 with the reference's
 * arithmetic; ROE's (gamma-1)/pow(a,2) uses the correctly rounded square.
 * Synchronous; allocates device memory for the batch. */
int amr_riemann(int32_t flux, int32_t dir_y, int32_t mag_field, double gamma, const double *wL, const double *wR,
                double *flux_out, int32_t *status, int64_t n);

/* ---- handing over a run (extension: no counterpart in the reference) -----
 * Instance `instance` of a created handle takes the quadtree and time state
 * of a run the caller owns, e.g. a reference run stopped after some step:
 * lp[last_active][8], icoord[last_active][2] and leafs[last_active] (the
 * meshblock records, defs.hpp:52-62), the reference's nbleafs counter, t, dt
 * and dt_next as amr_get_info reports them, and the step count.  Call it for
 * every instance instead of amr_init; then amr_upload U and Bi (and ff / gg,
 * whose low ghost face the next residual reads as the last stage left it,
 * main.cpp:150, for a bit-identical continuation) before stepping.  The tree
 * must have the structure admesh builds (IDs in range, father / son and
 * sibling links consistent, leaves sharing an edge at most one level apart);
 * anything else returns AMR_E_ARG and leaves the instance as it was. */
int amr_set_tree(amr_handle *h, int32_t instance, int32_t last_active, int32_t nb_leafs, const int32_t *lp,
                 const int32_t *icoord, const uint8_t *leafs, double t, double dt, double dt_next, int64_t steps);

/* ---- state exchange with host buffers ----------------------------------- */
/* Tree of one instance: lp[last_active][8], icoord[last_active][2], leafs[last_active] */
int amr_get_tree(amr_handle *h, int32_t instance, int32_t *lp, int32_t *icoord, uint8_t *leafs,
                 int32_t capacity);
/* field of blocks [0, last_active) of one instance as float64, layout
 * [block][var][j][i]; `count` = number of doubles the buffer holds */
int amr_download(amr_handle *h, int32_t instance, int32_t field, double *dst, int64_t count);
int amr_upload(amr_handle *h, int32_t instance, int32_t field, const double *src, int64_t count);

/* ---- measurement (no counterpart in the reference, which only has coarse
 * OpenMP wall-clock timers, main.cpp:124-256) ------------------------------ */
typedef struct amr_profile {
  int64_t launches;        /* kernels launched since the last enable/reset */
  int64_t stage_launches;  /* RK stages issued */
  double stage_ms;         /* CUDA-event time, on the launch stream, of each stage's dominant
                              kernel: the face-flux kernel (split stage) or the fused stage kernel */
  int64_t stage_cells;     /* leaf interior cells those launches updated */
  int64_t h2d_bytes;       /* host -> device bytes copied by the handle */
  int64_t d2h_bytes;
  double host_compile_ms;  /* host: leaf lists and ghost-fill compilation */
  double host_admesh_ms;   /* host: quadtree admesh */
  double wait_ms;          /* host: waiting for the device at step end */
  int64_t steps;
  double step_gpu_ms;      /* CUDA-event time, on the launch stream, of each step's device work
                              (its graph, or its kernel sequence when graphs are off) */
  double host_capture_ms;  /* host: capturing and instantiating / updating the step graph */
} amr_profile;
/* on != 0 starts recording events around the stage kernels; both reset the counters */
int amr_profile_enable(amr_handle *h, int32_t on);
int amr_profile_read(amr_handle *h, amr_profile *out);

/* Autotuner (no counterpart in the reference): times the candidate launch
 * schedules (fused or split RK stage; threads per CTA of the face-flux, cell
 * and ghost-fill kernels) on the handle's current state, `reps` probes each
 * (ghost fill + stage 1, which leaves U and Bi unchanged), and keeps the
 * fastest for later steps.  `report` (may be NULL) receives one line per
 * candidate, the chosen one marked with '*'. */
int amr_autotune(amr_handle *h, int32_t reps, char *report, size_t len);

/* ---- output and restart --------------------------------------------------
 * amr_save4py writes instance `inst` in the format of save4py
 * (savedata.cpp:7-46) to <dir>/<IC><id, 3 digits>t_<t>.dat: per leaf block a
 * "#" header line, then x, y, dx/2, dy/2, rho, u, v, w, p, Bx, By, Bz of
 * every interior cell in columns of width 16.  digits = 0 keeps the
 * reference's 6 significant digits; > 0 sets the precision (17 = exact;
 * above 9 digits the columns widen to digits + 9 characters).
 * The file name is copied to name_out (may be NULL).
 * amr_checkpoint_save / _load (extension): the whole handle (configurations,
 * counters, quadtrees, every field) in one binary file; load into a handle
 * created with the same configurations, in place of amr_init; the run then
 * continues bit for bit. */
int amr_save4py(amr_handle *h, int32_t inst, int32_t id, const char *dir, int32_t digits, char *name_out,
                size_t name_len);
int amr_checkpoint_save(amr_handle *h, const char *path);
int amr_checkpoint_load(amr_handle *h, const char *path);

/* ---- discrete adjoint of the frozen-mesh step (no counterpart in the
 * reference) ------------------------------------------------------------------
 * Reverse mode through whole time steps, with a checkpoint of (U, Bi) per
 * step and the step recomputed from it.  Supported: FP64, MUSCL with MC or
 * minmod, RUSA, nghosts 2, maxlevs 1 (frozen mesh) and dt_fixed > 0, else
 * AMR_E_UNSUPPORTED.
 *   amr_adjoint_enable(h, 1): clears the adjoint and the checkpoints; every
 *     later amr_step records one checkpoint (on = 0 drops them).
 *   amr_adjoint_seed: sets the adjoint (d loss / d field) of the current
 *     state, field AMR_FIELD_U or AMR_FIELD_BI, in amr_download's layout.
 *   amr_adjoint_step: reverses the last recorded step; the adjoint becomes
 *     that of the state before the step, and the state, t and the step count
 *     return to the checkpoint.  AMR_E_STATE when nothing is left to reverse.
 *   amr_adjoint_read: the current adjoint of U or BI (ghost entries are 0).
 *   amr_adjoint_recorded: steps that can still be reversed. */
int amr_adjoint_enable(amr_handle *h, int32_t on);
int amr_adjoint_seed(amr_handle *h, int32_t inst, int32_t field, const double *lam, int64_t count);
int amr_adjoint_step(amr_handle *h);
int amr_adjoint_read(amr_handle *h, int32_t inst, int32_t field, double *lam, int64_t count);
int amr_adjoint_recorded(amr_handle *h, int32_t *steps);

/* ---- allocation-free CFL reduction (no counterpart in the reference) ------
 * For callers that may not allocate device memory (inside a captured CUDA
 * graph, in allocator-free real-time loops, or in frameworks that own every
 * device allocation).  Same arithmetic as amr_cfl_dt (main.cpp:209-228) on the
 * caller's device arrays:
 *   U              [nblocks][8][16+2g][16+2g] float64 conserved state (leaf blocks)
 *   dxdy           [nblocks][2] float64 cell sizes (dx, dy) of each block
 *   dt_per_cfl_out one float64 on the device: the reference's `lambda`
 *                  (main.cpp:228), i.e. dt / CFL = min(1e6, min over blocks
 *                  of min(dx,dy) / max(|rho| + c_f,x, |u| + c_f,y)); NaN if a
 *                  block's wave speed is NaN (this variant has no pressure
 *                  trap)
 * The per-block scratch is a fixed file-scope device array of 65536 doubles
 * (512 KiB on every GPU that loads the library, kept until exit); nblocks
 * above 65536 returns AMR_E_TOO_LARGE.  The first call on a device looks up
 * that array's address and loads the entry point's kernels; make it before
 * any stream capture, and do not use the entry point after a cudaDeviceReset
 * in the same process (the looked-up address belongs to the old context).
 * Calls share the array, so calls that overlap on the GPU (different
 * streams) race: serialise them on one stream.  An error already pending in
 * the CUDA runtime is reported as AMR_E_CUDA and left for its owner.  Work
 * is enqueued on `cuda_stream`; the call does not synchronise. */
int amr_cfl_dt_static(const double *U, int32_t nblocks, int32_t nghosts, const double *dxdy, double gamma,
                      double *dt_per_cfl_out, void *cuda_stream);

#ifdef __cplusplus
}
#endif
#endif /* AMR2D_MHD_H */
