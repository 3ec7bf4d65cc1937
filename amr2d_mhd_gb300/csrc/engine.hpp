// The engine behind the C ABI: a pool of block slots resident on one GPU, the
// host quadtree of every instance, the compiled ghost fills, and the driver of
// one time step in the order of main.cpp:128-247.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <string>
#include <vector>

#include "../../include/amr2d_mhd.h"
#include "amr_common.h"
#include "ghost.cuh"
#include "ghost_compile.hpp"
#include "host_par.hpp"
#include "ic.hpp"
#include "launch.hpp"
#include "tree.hpp"

namespace amr {

// growable device buffer (contents are not preserved on growth)
struct DevBuf {
  void *p = nullptr;
  size_t bytes = 0;
  cudaError_t ensure(size_t n);
  void release();
  template <typename T> T *as() const { return static_cast<T *>(p); }
};

// pinned host buffer
struct HostBuf {
  void *p = nullptr;
  size_t bytes = 0;
  cudaError_t ensure(size_t n);
  void release();
  template <typename T> T *as() const { return static_cast<T *>(p); }
};

// engine-internal field ids of the adjoint arrays (transfers only)
constexpr int kFieldAdjU = 100, kFieldAdjB = 101;

struct Instance {
  amr_config cfg{};
  Tree tree;
  IcId ic = IC_INVALID;
  double gamma = 0, t_end = 0, cfl = 0;
  double t = 0, dt = 0, dtn = 0;
  int64_t count = 0;
  int64_t cell_updates = 0;
  bool done = false;
  bool handed = false;        // state given by amr_set_tree
  int limiter = 0;
  std::vector<int> slot;      // block ID -> physical slot, -1 if none yet
  double dx[16] = {0}, dy[16] = {0};
  int task_begin = 0, task_end = 0;  // this instance's leaves in the task list
  // compiled ghost fill of the current tree (snapshot rows numbered from 0)
  // and its range in the device program
  GhostProgram prog;
  uint64_t prog_version = ~0ull;
  bool prog_dirty = true;            // range not yet uploaded
  int64_t ops_off = 0, ops_cap = 0, snaps_off = 0, snaps_cap = 0;
  // device copy of slot[0, slotmap_n) for uploads and downloads (a block's
  // slot never changes once assigned)
  DevBuf d_slotmap;
  int slotmap_n = 0;
  explicit Instance(const TreeShape &s) : tree(s) {}
};

class Engine {
 public:
  Engine() = default;
  ~Engine();
  int create(const amr_config *cfgs, int n);
  int init();
  int step();
  int step_begin();                // rebuild + launch_step, no wait (amr_step_begin)
  int step_end();                  // finish_step of the step in flight (amr_step_end)
  bool step_pending() const { return step_pending_; }
  int run(int64_t max_steps);
  int info(int inst, amr_info *out);
  int set_stream(cudaStream_t s);
  // reference-function entry points (instance 0)
  int api_locate_bounds();
  int api_boundary(int field);
  int api_muscl2d_rk(int step);
  int api_ct2d(int step);
  int api_cfl_dt(double *lambda_min);
  int api_admesh();
  int api_criteria(double *grad, int32_t cap);
  int api_criteria_flags(uint8_t *iref, uint8_t *icoarse, int32_t cap);
  int api_admesh_marked(const uint8_t *iref, const uint8_t *icoarse, int32_t n);
  int api_set_tree(int q, int32_t last_active, int32_t nb_leafs, const int32_t *lp, const int32_t *icoord,
                   const uint8_t *leafs, double t, double dt, double dtn, int64_t steps);
  // host <-> device state
  int get_tree(int inst, int32_t *lp, int32_t *icoord, uint8_t *leafs, int32_t cap);
  int download(int inst, int field, double *dst, int64_t count);
  int upload(int inst, int field, const double *src, int64_t count);

  int profile_enable(bool on);
  // off: a step ends after the dt reduction, without main.cpp:246's admesh
  int set_remesh(bool on) {
    remesh_ = on;
    return 0;
  }
  int profile_read(amr_profile *out);

  // Times candidate launch schedules (fused or split stage, threads per CTA
  // of the face, cell and ghost kernels) on the current state with an
  // idempotent probe (ghost fill of U and Bi + stage 1 + the fill after it),
  // keeps the fastest and describes the trials in `report`.
  int autotune(int reps, char *report, size_t len);

  // checkpoint / restart and the savedata.cpp writer (checkpoint.cu)
  int checkpoint_save(const char *path);
  int checkpoint_load(const char *path);
  int save4py(int inst, int id, const char *dir, int digits, char *name_out, size_t name_len);

  // discrete adjoint of the frozen-mesh step (adjoint.cu)
  int adjoint_enable(bool on);
  int adjoint_seed(int inst, int field, const double *lam, int64_t count);
  int adjoint_read(int inst, int field, double *lam, int64_t count);
  int adjoint_step();
  int adjoint_recorded() const { return static_cast<int>(ckpt_meta_.size()); }

  std::string last_error;

 private:
  int fail(int code, const std::string &msg);
  int cuda_fail(cudaError_t e, const char *where);
  int check_device_error();
  int ensure_slots(int needed);
  int assign_slots(Instance &in);
  int rebuild();               // leaf tasks + ghost programs for the active set
  int upload_params();
  void fill_params_host();
  int enqueue_stage_sequence();
  int enqueue_step();              // params upload, stage sequence, dt kernels, result copies
  int launch_step();               // launch_step_work, bracketed by events when profiling
  int launch_step_work();          // enqueue_step directly or as a replayed CUDA graph
  int fill(std::initializer_list<std::pair<FillKind, int>> what);
  // the stage, CT and dt kernels; with `fuse` (or the FillPass arguments) the
  // kernels also gather the fill they consume and save the next one's
  // snapshots (fused fills, enqueue_stage_sequence)
  int stage(int step, const FillFuse *fuse = nullptr);
  int ct2d(int step, const FillPass *in = nullptr, const FillPass *out = nullptr, int emf_buf = 0, int bnew_buf = 0);
  int dt_crit(bool want_grad, const FillFuse *fuse = nullptr);
  // fused fills: a fill of `what` with its snapshots in rotating buffer `buf`
  FillPass fill_pass(std::initializer_list<std::pair<FillKind, int>> what, int buf, int tile_seg = -1);
  FillFuse fill_fuse(const FillPass *apply, const FillPass *save) const;
  int snap_only(const FillPass &p);    // a fill's snapshot pass as a launch of its own
  bool fused_fills() const { return fuse_fills_ && fuse_ok_; }
  int finish_step();
  struct AdmeshMarks {
    const uint8_t *ref, *crs;
  };
  int admesh_all(const std::vector<int> &which, const std::vector<std::vector<double>> *host_grad,
                 const AdmeshMarks *marks = nullptr);
  int xfer(Instance &in, int field, double *host, bool to_device);
  int checkpoint_read(const char *path);   // checkpoint_load's body
  void *field_ptr(int field) const;
  int field_nv(int field) const;
  bool field_f32(int field) const;

  std::vector<Instance> inst_;
  Method m_{};
  int ng_ = 2, n_ = 20, nn_ = 400;
  bool f32_ = false;
  bool split_ = true;              // stage as prim / faces / resid kernels (else fused k_stage)
  bool fuse_fills_ = true;         // AMR2D_FUSED_FILLS=0: every ghost fill as launches of its own
  bool fuse_ok_ = false;           // every active program is grouped by leaf block
  bool ct_coop_ = true;            // fused fills: CT2D as one cooperative launch (AMR2D_CT_COOP=0: three)
  // uploads / downloads: the scatter / gather kernel reads / writes the
  // caller's page-locked array itself instead of a copy through a staging
  // buffer (AMR2D_ZERO_COPY=0: always the copy)
  bool zero_copy_ = true;
  cudaStream_t stream_ = nullptr;
  bool own_stream_ = false;
  bool initialised_ = false;
  bool poisoned_ = false;

  // block pool
  int cap_slots_ = 0, used_slots_ = 0;
  void *U_ = nullptr, *Us_ = nullptr, *ff_ = nullptr, *gg_ = nullptr, *W_ = nullptr;
  double *Bi_ = nullptr, *Bis_ = nullptr, *EMF_ = nullptr;

  // active set and compiled programs
  std::vector<int> active_;        // instances stepping this step
  std::vector<uint64_t> built_version_;
  std::vector<int> built_active_;
  bool programs_valid_ = false;
  std::vector<LeafTask> tasks_;
  std::vector<int> task_blk_;      // block ID of each task
  // ghost fill of the active set: the instances' programs side by side, each
  // in a range padded with no-op entries so a changed tree re-uploads only
  // its own range
  int64_t nops_ = 0, nsnaps_ = 0, hole_ops_ = 0;
  int compile_programs();          // recompile changed instances (host threads)
  int layout_programs(bool relayout);
  DevBuf d_tasks_, d_params_, d_lambda_, d_grad_, d_err_, d_snap_, d_ops_, d_snaps_;
  DevBuf d_treeops_, d_stage_, d_ctr_;
  DevBuf d_snap3_;                 // fused fills: three rotating snapshot buffers
  DevBuf d_bar_;                   // grid barrier of the cooperative CT launch
  FillFuse dt_fuse_{};             // fused fills: the last fill of the step, gathered by the dt kernel
  HostBuf h_params_, h_lambda_, h_grad_, h_err_, h_ops_, h_snaps_, h_tasks_;
  std::vector<GhostCompiler *> gcs_;  // one per compile thread
  HostPool pool_;                      // host threads of the parallel loops (remesh, compile, layout)

  // CUDA graph of one step, re-captured when gen_ moves (tree, pool, profiling)
  bool graph_on_ = true;
  cudaStream_t cap_stream_ = nullptr;
  cudaGraphExec_t exec_ = nullptr;
  uint64_t gen_ = 1, captured_gen_ = 0;
  int graph_ev_used_ = 0;
  int64_t graph_launches_ = 0;
  bool capturing_ = false;

  // measurement
  bool prof_on_ = false;
  bool remesh_ = true;
  amr_profile prof_{};
  std::vector<cudaEvent_t> ev_;     // start/stop pairs of this step's stage launches
  int ev_used_ = 0;
  bool diffuse_any_ = false;  // some leaf task carries TASK_DIFFUSE
  bool step_pending_ = false; // step_begin launched a step that step_end has not finished
  cudaEvent_t step_ev_[2] = {nullptr, nullptr};  // brackets the step's device work (profiling)
  bool step_ev_pending_ = false;
  int64_t stage_cells_pending_ = 0;
  void prof_collect();

  // adjoint: checkpoints of (U, Bi) at the start of every recorded step, the
  // adjoint arrays and the tape of the step being reversed
  struct InstMeta { double t, dt, dtn; int64_t count, cell_updates; };
  struct Checkpoint { std::vector<InstMeta> meta; std::vector<int> active; };
  struct AdjSeg { FillKind kind; double *a; int nv; };
  bool adj_on_ = false;
  std::vector<Checkpoint> ckpt_meta_;
  std::vector<DevBuf> ckpt_;               // one buffer per recorded step
  size_t ckpt_slots_ = 0;                  // slots each checkpoint holds
  DevBuf a_U_, a_Us_, a_B_, a_Bs_, a_E_, a_F_, a_G_, a_C_[8], a_take_;
  DevBuf t_W1_, t_B1_, t_BisF_, t_UsPre_, t_BnewF_, t_UPre_;
  int adjoint_supported();
  int adjoint_alloc();
  int adjoint_record();                    // called by step() before the step
  int adjoint_recompute();
  int adjoint_sequence();
  int ghost_adj(std::initializer_list<AdjSeg> what);
  int ct2d_taped(int step);
  int adjoint_enqueue();                   // recompute + transposed step on stream_
  cudaGraphExec_t adj_exec_ = nullptr;     // the same, captured (re-captured when gen_ moves)
  uint64_t adj_gen_ = 0;
};

}  // namespace amr
