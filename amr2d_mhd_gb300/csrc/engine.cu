// Engine: device block pool, per-step orchestration and state exchange.
#include "engine.hpp"

#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <algorithm>
#include <atomic>
#include <chrono>
#include <initializer_list>
#include <mutex>
#include <string>
#include <thread>

#include "aux_kernels.cuh"
#include "host_par.hpp"
#include "stage_split.cuh"

namespace amr {

// ------------------------------------------------------------- buffers
cudaError_t DevBuf::ensure(size_t n) {
  if (n <= bytes && p) return cudaSuccess;
  release();
  size_t want = n < 256 ? 256 : n;
  cudaError_t e = cudaMalloc(&p, want);
  if (e != cudaSuccess) { p = nullptr; bytes = 0; return e; }
  bytes = want;
  return cudaSuccess;
}
void DevBuf::release() {
  if (p) cudaFree(p);
  p = nullptr;
  bytes = 0;
}
cudaError_t HostBuf::ensure(size_t n) {
  if (n <= bytes && p) return cudaSuccess;
  release();
  size_t want = n < 256 ? 256 : n;
  cudaError_t e = cudaMallocHost(&p, want);
  if (e != cudaSuccess) { p = nullptr; bytes = 0; return e; }
  bytes = want;
  return cudaSuccess;
}
void HostBuf::release() {
  if (p) cudaFreeHost(p);
  p = nullptr;
  bytes = 0;
}

namespace {
int lim_from_name(const char *s) {
  static const char *names[] = {"1st", "noSL", "minmod", "VanLeer", "Superbee", "MC", "Koren", "Cada3rd",
                                "WENO3", "WENO5"};
  if (!std::strcmp(s, "WENO2D")) return LIM_NOSL;  // slopelimiter.cpp:10
  for (int i = 0; i < 10; i++)
    if (!std::strcmp(s, names[i])) return i;
  return -1;
}
int flux_from_name(const char *s) {
  static const char *names[] = {"RUSA", "HLLE", "HLLC", "HLLD", "ROE"};
  for (int i = 0; i < 5; i++)
    if (!std::strcmp(s, names[i])) return i;
  return -1;
}
int map_dev_error(int code) {
  switch (code) {
    case DERR_PRESSURE: return AMR_E_PRESSURE;
    case DERR_HLLC: return AMR_E_HLLC;
    case DERR_TIMEOUT: return AMR_E_TIMEOUT;
    case DERR_PSI: return AMR_E_CT;
    default: return AMR_E_NAN;
  }
}
}  // namespace

Engine::~Engine() {
  if (stream_) cudaStreamSynchronize(stream_);
  for (void *p : {U_, Us_, ff_, gg_, W_}) if (p) cudaFree(p);
  for (double *p : {Bi_, Bis_, EMF_}) if (p) cudaFree(p);
  for (DevBuf *b : {&d_tasks_, &d_params_, &d_lambda_, &d_grad_, &d_err_, &d_snap_, &d_treeops_, &d_stage_,
                    &d_ctr_, &d_snap3_, &d_bar_})
    b->release();
  d_ops_.release();
  d_snaps_.release();
  for (DevBuf *b : {&a_U_, &a_Us_, &a_B_, &a_Bs_, &a_E_, &a_F_, &a_G_, &a_take_, &t_W1_, &t_B1_, &t_BisF_,
                    &t_UsPre_, &t_BnewF_, &t_UPre_})
    b->release();
  for (DevBuf &b : a_C_) b.release();
  for (Instance &in : inst_) in.d_slotmap.release();
  for (DevBuf &b : ckpt_) b.release();
  for (HostBuf *b : {&h_params_, &h_lambda_, &h_grad_, &h_err_, &h_ops_, &h_snaps_, &h_tasks_})
    b->release();
  if (own_stream_ && stream_) cudaStreamDestroy(stream_);
  if (exec_) cudaGraphExecDestroy(exec_);
  if (adj_exec_) cudaGraphExecDestroy(adj_exec_);
  if (cap_stream_) cudaStreamDestroy(cap_stream_);
  for (cudaEvent_t e : ev_) cudaEventDestroy(e);
  for (cudaEvent_t e : step_ev_)
    if (e) cudaEventDestroy(e);
  for (GhostCompiler *g : gcs_) delete g;
}

int Engine::fail(int code, const std::string &msg) {
  last_error = msg;
  if (code != AMR_E_ARG && code != AMR_E_CONFIG && code != AMR_E_STATE && code != AMR_E_UNSUPPORTED)
    poisoned_ = true;
  return code;
}

int Engine::cuda_fail(cudaError_t e, const char *where) {
  if (e == cudaErrorMemoryAllocation) return fail(AMR_E_OOM, std::string(where) + ": out of device memory");
  return fail(AMR_E_CUDA, std::string(where) + ": " + cudaGetErrorString(e));
}

#define CK(expr, where)                              \
  do {                                               \
    cudaError_t e_ = (expr);                         \
    if (e_ != cudaSuccess) return cuda_fail(e_, where); \
  } while (0)

// ------------------------------------------------------------- create
int Engine::create(const amr_config *cfgs, int n) {
  if (!cfgs || n <= 0) return fail(AMR_E_ARG, "no configuration");
  const amr_config &c0 = cfgs[0];
  for (int q = 0; q < n; q++) {
    const amr_config &c = cfgs[q];
    if (c.nx != NI || c.ny != NI) return fail(AMR_E_UNSUPPORTED, "blocks of 16 x 16 interior cells only");
    if (c.nvar != NVAR) return fail(AMR_E_CONFIG, "nvar must be 8 (MHD, meshblock.cpp:10-12)");
    if (c.nghosts != 2 && c.nghosts != 4) return fail(AMR_E_CONFIG, "nghosts must be 2 or 4");
    if (c.maxlevs < 1 || c.maxlevs > 12) return fail(AMR_E_CONFIG, "maxlevs out of range");
    if (c.nroots_x < 1 || c.nroots_y < 1) return fail(AMR_E_CONFIG, "nroots out of range");
    if (c.periodic && (c.nroots_x < 2 || c.nroots_y < 2))
      return fail(AMR_E_CONFIG, "a periodic box needs at least 2 x 2 root blocks");
    const int lim = lim_from_name(c.limiter), fl = flux_from_name(c.flux);
    if (lim < 0) return fail(AMR_E_CONFIG, std::string("invalid slope limiter '") + c.limiter + "'");
    if (fl < 0) return fail(AMR_E_CONFIG, std::string("no appropriate Riemann solver '") + c.flux + "'");
    if (fl == FLX_ROE) return fail(AMR_E_UNSUPPORTED, "ROE not ready with magnetic field (riemannS.cpp:39-40)");
    if (ic_from_name(c.ic) == IC_INVALID) return fail(AMR_E_CONFIG, std::string("no valid initial condition '") + c.ic + "'");
    if (lim == LIM_WENO5 && c.nghosts < 4) return fail(AMR_E_CONFIG, "WENO5 needs nghosts = 4");
    if (c.ct_type < 0 || c.ct_type > 2) return fail(AMR_E_CONFIG, "ct_type must be 1 (or 0) or 2");
    if (c.diffusion != 0 && c.diffusion != 1) return fail(AMR_E_CONFIG, "diffusion must be 0 or 1");
    // a batch shares the kernels: same method and block shape
    auto family = [](int l) { return l == LIM_WENO3 ? 1 : (l == LIM_WENO5 ? 2 : 0); };
    if (q > 0 && family(lim) != family(lim_from_name(c0.limiter)))
      return fail(AMR_E_CONFIG, "instances of a batch must share the reconstruction family");
    if (q > 0 && (fl != flux_from_name(c0.flux) || c.nghosts != c0.nghosts || c.precision != c0.precision))
      return fail(AMR_E_CONFIG, "instances of a batch must share flux, nghosts and precision");
  }
  const int lim0 = lim_from_name(c0.limiter);
  m_.ng = c0.nghosts;
  m_.recon = lim0 == LIM_WENO3 ? REC_WENO3 : (lim0 == LIM_WENO5 ? REC_WENO5 : REC_MUSCL);
  m_.flux = flux_from_name(c0.flux);
  m_.f32 = c0.precision == AMR_FP32 ? 1 : 0;
  if (!method_supported(m_)) return fail(AMR_E_UNSUPPORTED, "method not compiled");
  f32_ = m_.f32 != 0;
  if (const char *k = std::getenv("AMR2D_STAGE_KERNEL")) split_ = std::strcmp(k, "fused") != 0;
  if (const char *g = std::getenv("AMR2D_GRAPHS")) graph_on_ = std::strcmp(g, "0") != 0;
  if (const char *p = std::getenv("AMR2D_PDL")) m_.pdl = std::strcmp(p, "0") != 0 ? 1 : 0;
  if (const char *f = std::getenv("AMR2D_FUSED_FILLS")) fuse_fills_ = std::strcmp(f, "0") != 0;
  if (const char *f = std::getenv("AMR2D_CT_COOP")) ct_coop_ = std::strcmp(f, "0") != 0;
  if (const char *f = std::getenv("AMR2D_ZERO_COPY")) zero_copy_ = std::strcmp(f, "0") != 0;
  if (const char *f = std::getenv("AMR2D_FACE_KERNEL"))
    m_.persistent = !std::strcmp(f, "dynamic") ? 2 : (!std::strcmp(f, "persistent") ? 1 : 0);
  ng_ = m_.ng;
  n_ = NI + 2 * ng_;
  nn_ = n_ * n_;
  int ndev = 0;
  cudaError_t e = cudaGetDeviceCount(&ndev);
  if (e != cudaSuccess || ndev == 0) return fail(AMR_E_CUDA, "no CUDA device");
  CK(cudaStreamCreateWithFlags(&stream_, cudaStreamNonBlocking), "stream");
  own_stream_ = true;
  CK(cudaStreamCreateWithFlags(&cap_stream_, cudaStreamNonBlocking), "stream");
  inst_.reserve(n);
  for (int q = 0; q < n; q++) {
    const amr_config &c = cfgs[q];
    TreeShape s{NI, NI, c.nghosts, c.maxlevs, c.nroots_x, c.nroots_y, c.periodic != 0};
    inst_.emplace_back(s);
    Instance &in = inst_.back();
    in.cfg = c;
    in.ic = ic_from_name(c.ic);
    ic_params(in.ic, in.gamma, in.t_end);
    if (c.gamma > 0) in.gamma = c.gamma;
    if (c.t_end > 0) in.t_end = c.t_end;
    in.cfl = c.cfl;
    in.limiter = lim_from_name(c.limiter);
    // meshblock.cpp:87-96
    const int ni = NI;
    if (c.geometry == 0) {
      in.dx[0] = c.lenx / (static_cast<double>(c.nroots_x) * (ni - 1));
      in.dy[0] = c.leny / (static_cast<double>(c.nroots_y) * (ni - 1));
    } else {
      in.dx[0] = c.lenx / (static_cast<double>(c.nroots_x) * ni);
      in.dy[0] = c.leny / (static_cast<double>(c.nroots_y) * ni);
    }
    for (int l = 1; l < 16; l++) { in.dx[l] = in.dx[l - 1] / 2.; in.dy[l] = in.dy[l - 1] / 2.; }
    in.slot.assign(in.tree.maxblocks(), -1);
  }
  built_version_.assign(n, ~0ull);
  CK(d_err_.ensure(sizeof(DevError)), "alloc");
  CK(cudaMemsetAsync(d_err_.p, 0, sizeof(DevError), stream_), "memset");
  CK(d_ctr_.ensure(2 * sizeof(unsigned)), "alloc");   // k_faces_dyn's counters, zero between launches
  CK(cudaMemsetAsync(d_ctr_.p, 0, 2 * sizeof(unsigned), stream_), "memset");
  CK(d_bar_.ensure(2 * sizeof(unsigned)), "alloc");   // k_ct_coop's grid barrier (count, generation)
  CK(cudaMemsetAsync(d_bar_.p, 0, 2 * sizeof(unsigned), stream_), "memset");
  CK(h_err_.ensure(sizeof(DevError)), "alloc");
  CK(h_params_.ensure(sizeof(InstParams) * n), "alloc");
  CK(d_params_.ensure(sizeof(InstParams) * n), "alloc");
  return AMR_OK;
}

int Engine::set_stream(cudaStream_t s) {
  if (stream_) cudaStreamSynchronize(stream_);
  if (own_stream_ && stream_) cudaStreamDestroy(stream_);
  own_stream_ = false;
  stream_ = s;
  return AMR_OK;
}

void *Engine::field_ptr(int f) const {
  switch (f) {
    case AMR_FIELD_U: return U_;
    case AMR_FIELD_US: return Us_;
    case AMR_FIELD_FF: return ff_;
    case AMR_FIELD_GG: return gg_;
    case AMR_FIELD_BI: return Bi_;
    case AMR_FIELD_BIS: return Bis_;
    case AMR_FIELD_EMF: return EMF_;
    case kFieldAdjU: return a_U_.p;
    case kFieldAdjB: return a_B_.p;
    default: return nullptr;
  }
}
int Engine::field_nv(int f) const {
  if (f == AMR_FIELD_BI || f == AMR_FIELD_BIS || f == kFieldAdjB) return 2;
  if (f == AMR_FIELD_EMF) return 1;
  return 8;
}
bool Engine::field_f32(int f) const {
  return f32_ && (f == AMR_FIELD_U || f == AMR_FIELD_US || f == AMR_FIELD_FF || f == AMR_FIELD_GG);
}

// ------------------------------------------------------------- slots
int Engine::ensure_slots(int needed) {
  if (needed <= cap_slots_) return AMR_OK;
  int cap = cap_slots_ ? cap_slots_ : 64;
  while (cap < needed) cap *= 2;
  CK(cudaStreamSynchronize(stream_), "sync");
  const size_t cell = static_cast<size_t>(8) * nn_, face = static_cast<size_t>(2) * nn_, edge = nn_;
  const size_t se = f32_ ? sizeof(float) : sizeof(double);
  void **cells[5] = {&U_, &Us_, &ff_, &gg_, &W_};
  for (void **pp : cells) {
    void *np = nullptr;
    CK(cudaMalloc(&np, cap * cell * se), "pool alloc");
    CK(cudaMemsetAsync(np, 0, cap * cell * se, stream_), "pool memset");
    if (*pp) {
      CK(cudaMemcpyAsync(np, *pp, cap_slots_ * cell * se, cudaMemcpyDeviceToDevice, stream_), "pool copy");
      CK(cudaStreamSynchronize(stream_), "sync");
      cudaFree(*pp);
    }
    *pp = np;
  }
  double **dbl[3] = {&Bi_, &Bis_, &EMF_};
  const size_t per[3] = {face, face, edge};
  for (int q = 0; q < 3; q++) {
    double *np = nullptr;
    CK(cudaMalloc(&np, cap * per[q] * sizeof(double)), "pool alloc");
    CK(cudaMemsetAsync(np, 0, cap * per[q] * sizeof(double), stream_), "pool memset");
    if (*dbl[q]) {
      CK(cudaMemcpyAsync(np, *dbl[q], cap_slots_ * per[q] * sizeof(double), cudaMemcpyDeviceToDevice, stream_),
         "pool copy");
      CK(cudaStreamSynchronize(stream_), "sync");
      cudaFree(*dbl[q]);
    }
    *dbl[q] = np;
  }
  cap_slots_ = cap;
  gen_++;
  return AMR_OK;
}

int Engine::assign_slots(Instance &in) {
  for (int b = 0; b < in.tree.lastActive; b++)
    if (in.slot[b] < 0) in.slot[b] = used_slots_++;
  return ensure_slots(used_slots_);
}

// ------------------------------------------------------------- programs
// Recompiles the ghost fill of every active instance whose tree changed since
// its last compile, spread over host threads (one compiler each).
int Engine::compile_programs() {
  std::vector<int> todo;
  size_t blocks = 0;
  for (int a : active_)
    if (inst_[a].prog_version != inst_[a].tree.version) {
      todo.push_back(a);
      blocks += static_cast<size_t>(inst_[a].tree.lastActive);
    }
  if (todo.empty()) return AMR_OK;
  const size_t nth = host_threads(blocks);
  while (gcs_.size() < nth) gcs_.push_back(new GhostCompiler(n_, ng_));
  std::vector<std::vector<Bound>> bounds(nth);
  const std::string err = parallel_items(pool_, todo.size(), nth, [&](size_t w, size_t q) {
    Instance &in = inst_[todo[q]];
    in.tree.locate_bounds(bounds[w]);
    in.prog.clear();
    gcs_[w]->compile(in.tree, bounds[w], in.slot.data(), in.prog);
    in.prog_version = in.tree.version;
    in.prog_dirty = true;
  });
  if (!err.empty()) return fail(AMR_E_STATE, err);
  return AMR_OK;
}

namespace {
// grow a device buffer keeping its first `keep` bytes
cudaError_t grow_keep(DevBuf &b, size_t n, size_t keep, cudaStream_t s) {
  if (n <= b.bytes && b.p) return cudaSuccess;
  DevBuf nb;
  cudaError_t e = nb.ensure(n + n / 2);
  if (e != cudaSuccess) return e;
  if (b.p && keep) {
    e = cudaMemcpyAsync(nb.p, b.p, keep, cudaMemcpyDeviceToDevice, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) { nb.release(); return e; }
  }
  b.release();
  b = nb;
  return cudaSuccess;
}
cudaError_t grow_keep(HostBuf &b, size_t n, size_t keep) {
  if (n <= b.bytes && b.p) return cudaSuccess;
  HostBuf nb;
  cudaError_t e = nb.ensure(n + n / 2);
  if (e != cudaSuccess) return e;
  if (b.p && keep) std::memcpy(nb.p, b.p, keep);
  b.release();
  b = nb;
  return cudaSuccess;
}
}  // namespace

// Places every active instance's program in its own padded range of the
// device program (a pinned host mirror holds the whole layout) and uploads
// the ranges that changed.  A program that outgrows its range moves to the
// end and leaves a no-op hole; a full relayout compacts the holes once they
// are half of the program, and runs whenever the active set changes.
int Engine::layout_programs(bool relayout) {
  auto pad = [](int64_t n) { return n + n / 4 + 64; };
  std::vector<std::pair<int64_t, int64_t>> op_holes, snap_holes;
  int64_t o = nops_, sn = nsnaps_;
  if (!relayout) {
    for (int a : active_) {
      Instance &in = inst_[a];
      if (static_cast<int64_t>(in.prog.ops.size()) <= in.ops_cap &&
          static_cast<int64_t>(in.prog.snaps.size()) <= in.snaps_cap)
        continue;
      op_holes.emplace_back(in.ops_off, in.ops_cap);
      snap_holes.emplace_back(in.snaps_off, in.snaps_cap);
      hole_ops_ += in.ops_cap;
      in.ops_off = o;
      in.ops_cap = pad(static_cast<int64_t>(in.prog.ops.size()));
      o += in.ops_cap;
      in.snaps_off = sn;
      in.snaps_cap = pad(static_cast<int64_t>(in.prog.snaps.size()));
      sn += in.snaps_cap;
      in.prog_dirty = true;
    }
    if (hole_ops_ > o / 2) relayout = true;
  }
  if (relayout) {
    o = sn = 0;
    op_holes.clear();
    snap_holes.clear();
    hole_ops_ = 0;
    for (int a : active_) {
      Instance &in = inst_[a];
      in.ops_off = o;
      in.ops_cap = pad(static_cast<int64_t>(in.prog.ops.size()));
      o += in.ops_cap;
      in.snaps_off = sn;
      in.snaps_cap = pad(static_cast<int64_t>(in.prog.snaps.size()));
      sn += in.snaps_cap;
      in.prog_dirty = true;
    }
  }
  const size_t keep_o = relayout ? 0 : sizeof(GhostOp) * nops_;
  const size_t keep_s = relayout ? 0 : sizeof(GhostSnap) * nsnaps_;
  CK(grow_keep(d_ops_, sizeof(GhostOp) * o, keep_o, stream_), "alloc");
  CK(grow_keep(d_snaps_, sizeof(GhostSnap) * sn, keep_s, stream_), "alloc");
  CK(grow_keep(h_ops_, sizeof(GhostOp) * o, keep_o), "alloc");
  CK(grow_keep(h_snaps_, sizeof(GhostSnap) * sn, keep_s), "alloc");
  nops_ = o;
  nsnaps_ = sn;
  CK(d_snap_.ensure(sizeof(double) * 8 * (static_cast<size_t>(kMaxSeg) * nsnaps_ + 1)), "alloc");
  CK(d_snap3_.ensure(sizeof(double) * 8 * (3 * static_cast<size_t>(kMaxSeg) * nsnaps_ + 1)), "alloc");
  GhostOp *ho = h_ops_.as<GhostOp>();
  GhostSnap *hs = h_snaps_.as<GhostSnap>();
  const GhostOp nop{0, 0, 0, 0, GOP_NOP, {0, 0, 0}};
  const GhostSnap nosnap{-1, 0};
  // ranges to upload: holes (filled with no-ops) and the dirty programs
  std::vector<std::pair<int64_t, int64_t>> up_ops(op_holes), up_snaps(snap_holes);
  for (const auto &h : op_holes)
    for (int64_t q = 0; q < h.second; q++) ho[h.first + q] = nop;
  for (const auto &h : snap_holes)
    for (int64_t q = 0; q < h.second; q++) hs[h.first + q] = nosnap;
  std::vector<int> dirty;
  size_t blocks = 0;
  for (int a : active_)
    if (inst_[a].prog_dirty) {
      dirty.push_back(a);
      blocks += static_cast<size_t>(inst_[a].tree.lastActive);
      up_ops.emplace_back(inst_[a].ops_off, inst_[a].ops_cap);
      up_snaps.emplace_back(inst_[a].snaps_off, inst_[a].snaps_cap);
    }
  parallel_items(pool_, dirty.size(), host_threads(blocks), [&](size_t, size_t q) {
    Instance &in = inst_[dirty[q]];
    const int64_t no = static_cast<int64_t>(in.prog.ops.size()), ns = static_cast<int64_t>(in.prog.snaps.size());
    GhostOp *d = ho + in.ops_off;
    for (int64_t k = 0; k < no; k++) {
      d[k] = in.prog.ops[k];
      if (d[k].type == GOP_SNAP || d[k].type == GOP_SFINE) d[k].src_slot += static_cast<int32_t>(in.snaps_off);
    }
    for (int64_t k = no; k < in.ops_cap; k++) d[k] = nop;
    if (ns) std::memcpy(hs + in.snaps_off, in.prog.snaps.data(), sizeof(GhostSnap) * ns);
    for (int64_t k = ns; k < in.snaps_cap; k++) hs[in.snaps_off + k] = nosnap;
    in.prog_dirty = false;
  });
  // one copy per run of adjacent ranges
  int64_t bytes = 0;
  auto upload = [&](std::vector<std::pair<int64_t, int64_t>> &r, bool ops) -> int {
    std::sort(r.begin(), r.end());
    const size_t sz = ops ? sizeof(GhostOp) : sizeof(GhostSnap);
    char *dbase = static_cast<char *>(ops ? d_ops_.p : d_snaps_.p);
    const char *hbase = ops ? reinterpret_cast<const char *>(ho) : reinterpret_cast<const char *>(hs);
    for (size_t q = 0; q < r.size();) {
      const int64_t off = r[q].first;
      int64_t end = off + r[q].second;
      size_t k = q + 1;
      while (k < r.size() && r[k].first <= end) { end = std::max(end, r[k].first + r[k].second); k++; }
      if (end > off) {
        CK(cudaMemcpyAsync(dbase + sz * off, hbase + sz * off, sz * (end - off), cudaMemcpyHostToDevice, stream_),
           "h2d");
        bytes += static_cast<int64_t>(sz * (end - off));
      }
      q = k;
    }
    return AMR_OK;
  };
  if (int rc = upload(up_ops, true)) return rc;
  if (int rc = upload(up_snaps, false)) return rc;
  prof_.h2d_bytes += bytes;
  return AMR_OK;
}

int Engine::rebuild() {
  bool need = !programs_valid_ || built_active_ != active_;
  for (int a : active_)
    if (built_version_[a] != inst_[a].tree.version) need = true;
  if (!need) return AMR_OK;
  gen_++;
  const auto t0 = std::chrono::steady_clock::now();
  const bool relayout = !programs_valid_ || built_active_ != active_;
  if (int rc = compile_programs()) return rc;
  tasks_.clear();
  task_blk_.clear();
  diffuse_any_ = false;
  for (int a : active_) {
    Instance &in = inst_[a];
    in.task_begin = static_cast<int>(tasks_.size());
    for (int nb = 0; nb < in.tree.lastActive; nb++) {
      if (!in.tree.leafs[nb]) continue;
      const int lev = in.tree.lp[nb][0];
      const int flags = in.cfg.diffusion && lev >= in.cfg.maxlevs - 2 ? TASK_DIFFUSE : 0;
      diffuse_any_ |= flags != 0;
      tasks_.push_back(LeafTask{in.slot[nb], a, in.dx[lev], in.dy[lev], exact_reciprocal(in.dx[lev]),
                                exact_reciprocal(in.dy[lev]), 1. / in.dx[lev], 1. / in.dy[lev], flags, 0, 0, 0, 0,
                                0});
      task_blk_.push_back(nb);
    }
    in.task_end = static_cast<int>(tasks_.size());
    built_version_[a] = in.tree.version;
  }
  built_active_ = active_;
  if (int rc = layout_programs(relayout)) return rc;
  // each leaf's share of its instance's program (the program is grouped by
  // block; the fused fills need every written or saved block to be a leaf)
  fuse_ok_ = true;
  for (int a : active_) fuse_ok_ = fuse_ok_ && inst_[a].prog.by_block;
  if (fuse_ok_)
    for (size_t k = 0; k < tasks_.size(); k++) {
      const Instance &in = inst_[tasks_[k].inst];
      const int nb = task_blk_[k];
      LeafTask &t = tasks_[k];
      t.op_begin = static_cast<int>(in.ops_off) + in.prog.op_start[nb];
      t.op_count = in.prog.op_start[nb + 1] - in.prog.op_start[nb];
      t.snap_begin = static_cast<int>(in.snaps_off) + in.prog.snap_start[nb];
      t.snap_count = in.prog.snap_start[nb + 1] - in.prog.snap_start[nb];
    }
  const size_t nt = tasks_.size();
  CK(d_tasks_.ensure(sizeof(LeafTask) * nt), "alloc");
  CK(h_tasks_.ensure(sizeof(LeafTask) * nt), "alloc");
  std::memcpy(h_tasks_.p, tasks_.data(), sizeof(LeafTask) * nt);
  CK(cudaMemcpyAsync(d_tasks_.p, h_tasks_.p, sizeof(LeafTask) * nt, cudaMemcpyHostToDevice, stream_), "h2d");
  CK(d_lambda_.ensure(sizeof(double) * nt), "alloc");
  CK(d_grad_.ensure(sizeof(double) * nt), "alloc");
  CK(h_lambda_.ensure(sizeof(double) * nt), "alloc");
  CK(h_grad_.ensure(sizeof(double) * nt), "alloc");
  // the pinned mirrors above must not change before the copies have run
  CK(cudaStreamSynchronize(stream_), "sync");
  programs_valid_ = true;
  prof_.h2d_bytes += static_cast<int64_t>(sizeof(LeafTask) * nt);
  prof_.host_compile_ms += std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
  return AMR_OK;
}

void Engine::fill_params_host() {
  InstParams *p = h_params_.as<InstParams>();
  for (size_t q = 0; q < inst_.size(); q++) {
    p[q].gamma = inst_[q].gamma;
    p[q].dt = inst_[q].dt;
    p[q].limiter = inst_[q].limiter;
    p[q].ct_type = inst_[q].cfg.ct_type == 2 ? 2 : 1;
  }
}

int Engine::upload_params() {
  fill_params_host();
  InstParams *p = h_params_.as<InstParams>();
  CK(cudaMemcpyAsync(d_params_.p, p, sizeof(InstParams) * inst_.size(), cudaMemcpyHostToDevice, stream_), "h2d");
  prof_.h2d_bytes += sizeof(InstParams) * inst_.size();
  return AMR_OK;
}

// ------------------------------------------------------------- kernels
int Engine::fill(std::initializer_list<std::pair<FillKind, int>> what) {
  GhostLaunch g{};
  g.ops = d_ops_.as<GhostOp>();
  g.snaps = d_snaps_.as<GhostSnap>();
  g.nops = static_cast<int>(nops_);
  g.nsnaps = static_cast<int>(nsnaps_);
  int q = 0;
  for (const auto &w : what) {
    GhostSeg &s = g.seg[q++];
    s.field = field_ptr(w.second);
    s.nv = field_nv(w.second);
    s.kind = w.first;
    s.f32 = field_f32(w.second) ? 1 : 0;
  }
  g.nseg = q;
  g.snapbuf = d_snap_.as<double>();
  CK(launch_ghost(m_, g, stream_), "ghost fill");
  prof_.launches += (g.nsnaps > 0) + (g.nops > 0);
  return AMR_OK;
}

FillPass Engine::fill_pass(std::initializer_list<std::pair<FillKind, int>> what, int buf, int tile_seg) {
  FillPass p{};
  int q = 0;
  for (const auto &w : what) {
    GhostSeg &g = p.seg[q++];
    g.field = field_ptr(w.second);
    g.nv = field_nv(w.second);
    g.kind = w.first;
    g.f32 = field_f32(w.second) ? 1 : 0;
    p.rows += g.nv;
  }
  p.nseg = q;
  p.tile_seg = tile_seg;
  p.snapbuf = d_snap3_.as<double>() + static_cast<size_t>(buf) * kMaxSeg * nsnaps_ * 8;
  return p;
}

FillFuse Engine::fill_fuse(const FillPass *apply, const FillPass *save) const {
  FillFuse f{};
  f.ops = d_ops_.as<GhostOp>();
  f.snaps = d_snaps_.as<GhostSnap>();
  f.nsnaps = static_cast<int>(nsnaps_);
  if (apply) f.apply = *apply;
  if (save) f.save = *save;
  return f;
}

int Engine::snap_only(const FillPass &p) {
  if (nsnaps_ == 0) return AMR_OK;
  GhostLaunch g{};
  g.ops = d_ops_.as<GhostOp>();
  g.snaps = d_snaps_.as<GhostSnap>();
  g.nops = 0;
  g.nsnaps = static_cast<int>(nsnaps_);
  for (int q = 0; q < p.nseg; q++) g.seg[q] = p.seg[q];
  g.nseg = p.nseg;
  g.snapbuf = p.snapbuf;
  CK(launch_ghost(m_, g, stream_), "ghost snapshots");
  prof_.launches += 1;
  return AMR_OK;
}

int Engine::stage(int step, const FillFuse *fuse) {
  // profiling events bracket the dominant kernel: the face-flux kernel of the
  // split stage, or the fused stage kernel
  auto ev_begin = [&]() -> int {
    if (!prof_on_) return AMR_OK;
    while (ev_.size() < static_cast<size_t>(ev_used_ + 2)) {
      cudaEvent_t e;
      CK(cudaEventCreate(&e), "event");
      ev_.push_back(e);
    }
    // inside a graph capture the events must be external nodes to be timed
    CK(cudaEventRecordWithFlags(ev_[ev_used_], stream_, capturing_ ? cudaEventRecordExternal : 0), "event");
    return AMR_OK;
  };
  auto ev_end = [&]() -> int {
    if (!prof_on_) return AMR_OK;
    CK(cudaEventRecordWithFlags(ev_[ev_used_ + 1], stream_, capturing_ ? cudaEventRecordExternal : 0), "event");
    ev_used_ += 2;
    return AMR_OK;
  };
  const int n = static_cast<int>(tasks_.size());
  if (split_) {
    SplitArgs a{};
    a.tasks = d_tasks_.as<LeafTask>();
    a.inst = d_params_.as<InstParams>();
    a.qin = step == 1 ? U_ : Us_;
    a.qout = step == 1 ? Us_ : U_;
    a.W = W_;
    a.B = step == 1 ? Bi_ : Bis_;
    a.ff = ff_;
    a.gg = gg_;
    a.err = d_err_.as<DevError>();
    a.ctr = d_ctr_.as<unsigned>();
    a.step = step;
    a.ntasks = n;
    if (fuse) a.fuse = *fuse;
    CK(launch_prim(m_, a, stream_), "prim kernel");
    if (int rc = ev_begin()) return rc;
    CK(launch_faces(m_, a, stream_), "face kernel");
    if (int rc = ev_end()) return rc;
    CK(launch_resid(m_, a, stream_), "residual kernel");
    prof_.launches += 3;
  } else {
    StageArgs a{};
    a.tasks = d_tasks_.as<LeafTask>();
    a.inst = d_params_.as<InstParams>();
    a.qin = step == 1 ? U_ : Us_;
    a.qout = step == 1 ? Us_ : U_;
    a.B = step == 1 ? Bi_ : Bis_;
    a.ff = ff_;
    a.gg = gg_;
    a.err = d_err_.as<DevError>();
    a.ctr = d_ctr_.as<unsigned>();
    a.step = step;
    a.ntasks = n;
    if (fuse) a.fuse = *fuse;
    if (int rc = ev_begin()) return rc;
    CK(launch_stage(m_, a, n, stream_), "stage kernel");
    if (int rc = ev_end()) return rc;
    prof_.launches += 1;
  }
  if (step == 2 && diffuse_any_) {  // main.cpp:190-193, after each block's stage-2 update
    CtArgs d{};
    d.tasks = d_tasks_.as<LeafTask>();
    d.q = U_;
    CK(launch_diffuse(m_, d, n, stream_), "diffusion kernel");
    prof_.launches += 1;
  }
  prof_.stage_launches += 1;
  stage_cells_pending_ += static_cast<int64_t>(n) * NI * NI;
  return AMR_OK;
}

int Engine::autotune(int reps, char *report, size_t len) {
  if (!initialised_) return fail(AMR_E_STATE, "amr_init has not been called");
  if (poisoned_) return fail(AMR_E_STATE, "engine stopped by an earlier error: " + last_error);
  if (reps < 1) reps = 1;
  active_.clear();
  for (size_t q = 0; q < inst_.size(); q++)
    if (!inst_[q].done) active_.push_back(static_cast<int>(q));
  if (active_.empty()) return fail(AMR_E_STATE, "no active instance to tune on");
  if (int rc = rebuild()) return rc;
  if (int rc = upload_params()) return rc;
  const bool prof = prof_on_;
  prof_on_ = false;
  struct Cand { bool split; int fb, cb, gb, pers; float ms; };
  std::vector<Cand> cands;
  for (int gb : {128, 256, 512}) {
    cands.push_back({false, 128, 256, gb, 0, 0.f});
    cands.push_back({false, 128, 256, gb, 2, 0.f});   // fused, persistent over the leaf list
    for (int pers : {0, 1, 2})
      for (int fb : {64, 128})
        for (int cb : {256, 512}) cands.push_back({true, fb, cb, gb, pers, 0.f});
  }
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  CK(cudaEventCreate(&e0), "event");
  CK(cudaEventCreate(&e1), "event");
  auto probe = [&]() -> int {
    if (fused_fills()) {  // the step's form: snapshots, then the stage with the fill inside
      const FillPass f1 = fill_pass({{FILL_CC, AMR_FIELD_U}, {FILL_FC, AMR_FIELD_BI}}, 0, 0);
      const FillPass f2 = fill_pass({{FILL_FC, AMR_FIELD_BI}, {FILL_FC, AMR_FIELD_FF}, {FILL_FC, AMR_FIELD_GG}}, 1);
      if (int rc = snap_only(f1)) return rc;
      const FillFuse s1 = fill_fuse(&f1, &f2);
      return stage(1, &s1);
    }
    if (int rc = fill({{FILL_CC, AMR_FIELD_U}, {FILL_FC, AMR_FIELD_BI}})) return rc;
    if (int rc = stage(1)) return rc;
    return fill({{FILL_FC, AMR_FIELD_BI}, {FILL_FC, AMR_FIELD_FF}, {FILL_FC, AMR_FIELD_GG}});
  };
  int rc = AMR_OK;
  const Method keep = m_;
  const bool keep_split = split_;
  for (Cand &c : cands) {
    split_ = c.split;
    m_.faces_block = c.fb;
    m_.cell_block = c.cb;
    m_.ghost_block = c.gb;
    m_.persistent = c.pers;
    if ((rc = probe())) break;  // warm-up
    cudaEventRecord(e0, stream_);
    for (int r = 0; r < reps && !rc; r++) rc = probe();
    cudaEventRecord(e1, stream_);
    cudaError_t e = cudaEventSynchronize(e1);
    if (e != cudaSuccess) { rc = cuda_fail(e, "autotune"); break; }
    cudaEventElapsedTime(&c.ms, e0, e1);
    c.ms /= static_cast<float>(reps);
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  prof_on_ = prof;
  stage_cells_pending_ = 0;
  if (rc) { m_ = keep; split_ = keep_split; return rc; }
  if (int r2 = check_device_error()) return r2;
  const Cand *best = &cands[0];
  for (const Cand &c : cands)
    if (c.ms < best->ms) best = &c;
  split_ = best->split;
  m_.faces_block = best->fb;
  m_.cell_block = best->cb;
  m_.ghost_block = best->gb;
  m_.persistent = best->pers;
  gen_++;  // the captured step uses the chosen launches
  if (report && len) {
    std::string s;
    char line[160];
    for (const Cand &c : cands) {
      std::snprintf(line, sizeof line, "%s%s faces %d%s cells %d ghosts %d: %.4f ms\n", &c == best ? "* " : "  ",
                    c.split ? "split" : "fused", c.fb, c.pers == 2 ? " dynamic" : (c.pers ? " persistent" : ""), c.cb,
                    c.gb, c.ms);  // fused + dynamic: k_stage_dyn
      s += line;
    }
    std::strncpy(report, s.c_str(), len - 1);
    report[len - 1] = '\0';
  }
  return AMR_OK;
}

// CT2D.cpp:11-124: EMF, its ghost fill, the face update, its ghost fill and
// the cell-centred B / energy correction.  With `in` (fused fills) the EMF
// kernel gathers the fill `in`, the fills of the EMF and of the new face field
// run inside the next kernel (snapshots in rotating buffers emf_buf and
// bnew_buf), and the cell kernel saves the snapshots of `out`.
int Engine::ct2d(int step, const FillPass *in, const FillPass *out, int emf_buf, int bnew_buf) {
  CtArgs a{};
  a.tasks = d_tasks_.as<LeafTask>();
  a.inst = d_params_.as<InstParams>();
  a.ff = ff_;
  a.gg = gg_;
  a.EMF = EMF_;
  a.Bsrc = step == 1 ? Bi_ : Bis_;
  a.Bnew = step == 1 ? Bis_ : Bi_;
  a.q = step == 1 ? Us_ : U_;
  a.err = d_err_.as<DevError>();
  a.step = step;
  const int n = static_cast<int>(tasks_.size());
  a.ntasks = n;
  if (in) {
    const FillPass emf = fill_pass({{FILL_EC, AMR_FIELD_EMF}}, emf_buf);
    const FillPass bnew = fill_pass({{FILL_FC, step == 1 ? AMR_FIELD_BIS : AMR_FIELD_BI}}, bnew_buf);
    if (ct_coop_) {  // one cooperative launch, grid barriers between the phases
      CK(launch_ct_coop(m_, a, fill_fuse(in, &emf), fill_fuse(&emf, &bnew), fill_fuse(&bnew, out),
                        d_bar_.as<unsigned>(), stream_), "ct kernel");
      prof_.launches += 1;
      return AMR_OK;
    }
    a.fuse = fill_fuse(in, &emf);
    CK(launch_ct_emf(m_, a, n, stream_), "ct emf");
    a.fuse = fill_fuse(&emf, &bnew);
    CK(launch_ct_face(m_, a, n, stream_), "ct face");
    a.fuse = fill_fuse(&bnew, out);
    CK(launch_ct_cell(m_, a, n, stream_), "ct cell");
    prof_.launches += 3;
    return AMR_OK;
  }
  CK(launch_ct_emf(m_, a, n, stream_), "ct emf");
  if (int rc = fill({{FILL_EC, AMR_FIELD_EMF}})) return rc;
  CK(launch_ct_face(m_, a, n, stream_), "ct face");
  if (int rc = fill({{FILL_FC, step == 1 ? AMR_FIELD_BIS : AMR_FIELD_BI}})) return rc;
  CK(launch_ct_cell(m_, a, n, stream_), "ct cell");
  prof_.launches += 3;
  return AMR_OK;
}

// primitive state of U (with the pressure / NaN traps of U2W("main")) and
// the per-leaf wave-speed maximum and refinement criterion, in one kernel
int Engine::dt_crit(bool want_grad, const FillFuse *fuse) {
  DtArgs a{};
  a.tasks = d_tasks_.as<LeafTask>();
  a.inst = d_params_.as<InstParams>();
  a.U = U_;
  a.lambda = d_lambda_.as<double>();
  a.grad = d_grad_.as<double>();
  a.err = d_err_.as<DevError>();
  a.want_grad = want_grad ? 1 : 0;
  if (fuse) a.fuse = *fuse;
  CK(launch_dt_cell(m_, a, static_cast<int>(tasks_.size()), stream_), "dt kernel");
  prof_.launches += 1;
  return AMR_OK;
}

// main.cpp:129-202: ghost fills, stage 1 with CT, stage 2 with CT.  With
// fused fills the nine fills of the step run inside the kernels that consume
// them (the dt kernel takes the last), each kernel saving the next fill's
// snapshots; the first fill's snapshots are a launch of their own.  Snapshot
// buffers rotate over three, so that a kernel never writes the buffer it
// reads.
int Engine::enqueue_stage_sequence() {
  int rc;
  if (fused_fills()) {
    const FillPass f1 = fill_pass({{FILL_CC, AMR_FIELD_U}, {FILL_FC, AMR_FIELD_BI}}, 0, 0);
    const FillPass f2 = fill_pass({{FILL_FC, AMR_FIELD_BI}, {FILL_FC, AMR_FIELD_FF}, {FILL_FC, AMR_FIELD_GG}}, 1);
    const FillPass f5 = fill_pass({{FILL_CC, AMR_FIELD_US}}, 1, 0);
    const FillPass f6 = fill_pass({{FILL_FC, AMR_FIELD_FF}, {FILL_FC, AMR_FIELD_GG}}, 2);
    const FillPass f9 = fill_pass({{FILL_CC, AMR_FIELD_U}}, 2);
    if ((rc = snap_only(f1))) return rc;
    const FillFuse s1 = fill_fuse(&f1, &f2);
    if ((rc = stage(1, &s1))) return rc;
    if ((rc = ct2d(1, &f2, &f5, 2, 0))) return rc;     // EMF fill in buffer 2, Bis fill in 0
    const FillFuse s2 = fill_fuse(&f5, &f6);
    if ((rc = stage(2, &s2))) return rc;
    if ((rc = ct2d(2, &f6, &f9, 0, 1))) return rc;     // EMF fill in buffer 0, Bi fill in 1
    dt_fuse_ = fill_fuse(&f9, nullptr);
    return AMR_OK;
  }
  dt_fuse_ = FillFuse{};
  if ((rc = fill({{FILL_CC, AMR_FIELD_U}, {FILL_FC, AMR_FIELD_BI}}))) return rc;
  if ((rc = stage(1))) return rc;
  if ((rc = fill({{FILL_FC, AMR_FIELD_BI}, {FILL_FC, AMR_FIELD_FF}, {FILL_FC, AMR_FIELD_GG}}))) return rc;
  if ((rc = ct2d(1))) return rc;
  if ((rc = fill({{FILL_CC, AMR_FIELD_US}}))) return rc;
  if ((rc = stage(2))) return rc;
  if ((rc = fill({{FILL_FC, AMR_FIELD_FF}, {FILL_FC, AMR_FIELD_GG}}))) return rc;
  if ((rc = ct2d(2))) return rc;
  if ((rc = fill({{FILL_CC, AMR_FIELD_U}}))) return rc;
  return AMR_OK;
}

int Engine::enqueue_step() {
  if (int rc = upload_params()) return rc;
  if (int rc = enqueue_stage_sequence()) return rc;
  bool any_amr = false;
  for (int a : active_) any_amr |= inst_[a].cfg.maxlevs > 1;
  if (int rc = dt_crit(any_amr, dt_fuse_.apply.nseg ? &dt_fuse_ : nullptr)) return rc;
  const size_t nt = tasks_.size();
  CK(cudaMemcpyAsync(h_lambda_.p, d_lambda_.p, sizeof(double) * nt, cudaMemcpyDeviceToHost, stream_), "d2h");
  CK(cudaMemcpyAsync(h_grad_.p, d_grad_.p, sizeof(double) * nt, cudaMemcpyDeviceToHost, stream_), "d2h");
  return AMR_OK;
}

int Engine::launch_step() {
  if (prof_on_) {
    for (cudaEvent_t &e : step_ev_)
      if (!e) CK(cudaEventCreate(&e), "event");
    CK(cudaEventRecord(step_ev_[0], stream_), "event");
  }
  if (int rc = launch_step_work()) return rc;
  if (prof_on_) {
    CK(cudaEventRecord(step_ev_[1], stream_), "event");
    step_ev_pending_ = true;
  }
  return AMR_OK;
}

int Engine::launch_step_work() {
  const int64_t launches0 = prof_.launches;
  if (!graph_on_) return enqueue_step();
  if (!exec_ || captured_gen_ != gen_) {
    const auto t0 = std::chrono::steady_clock::now();
    // capture on a private stream; the graph is then launched on stream_
    cudaStream_t user = stream_;
    stream_ = cap_stream_;
    const int ev0 = ev_used_;
    // events are created outside the capture
    if (prof_on_)
      while (ev_.size() < static_cast<size_t>(ev0 + 4)) {
        cudaEvent_t e;
        CK(cudaEventCreate(&e), "event");
        ev_.push_back(e);
      }
    cudaError_t e = cudaStreamBeginCapture(cap_stream_, cudaStreamCaptureModeRelaxed);
    if (e != cudaSuccess) { stream_ = user; return cuda_fail(e, "graph capture"); }
    capturing_ = true;
    int rc = enqueue_step();
    capturing_ = false;
    cudaGraph_t g = nullptr;
    e = cudaStreamEndCapture(cap_stream_, &g);
    stream_ = user;
    if (rc) { if (g) cudaGraphDestroy(g); return rc; }
    if (e != cudaSuccess) return cuda_fail(e, "graph capture");
    graph_ev_used_ = ev_used_ - ev0;
    ev_used_ = ev0;
    bool updated = false;
    if (exec_) {
      cudaGraphExecUpdateResultInfo info;
      updated = cudaGraphExecUpdate(exec_, g, &info) == cudaSuccess;
      if (!updated) {
        cudaGetLastError();
        cudaGraphExecDestroy(exec_);
        exec_ = nullptr;
      }
    }
    if (!updated) {
      e = cudaGraphInstantiate(&exec_, g, 0);
      if (e != cudaSuccess) { cudaGraphDestroy(g); return cuda_fail(e, "graph instantiate"); }
    }
    cudaGraphDestroy(g);
    captured_gen_ = gen_;
    graph_launches_ = prof_.launches - launches0;
    prof_.host_capture_ms += std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
  } else {
    fill_params_host();  // the graph's first node copies these to the device
    prof_.launches += graph_launches_;
    prof_.stage_launches += 2;
    stage_cells_pending_ += 2 * static_cast<int64_t>(tasks_.size()) * NI * NI;
    prof_.h2d_bytes += sizeof(InstParams) * inst_.size();
  }
  ev_used_ += graph_ev_used_;
  CK(cudaGraphLaunch(exec_, stream_), "graph launch");
  return AMR_OK;
}

int Engine::check_device_error() {
  CK(cudaMemcpyAsync(h_err_.p, d_err_.p, sizeof(DevError), cudaMemcpyDeviceToHost, stream_), "d2h");
  prof_.d2h_bytes += sizeof(DevError);
  const auto w0 = std::chrono::steady_clock::now();
  CK(cudaStreamSynchronize(stream_), "sync");
  prof_.wait_ms += std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - w0).count();
  prof_collect();
  const DevError &e = *h_err_.as<DevError>();
  if (e.code != 0) {
    char msg[256];
    std::snprintf(msg, sizeof msg, "device check failed (code %d) at slot %d cell (%d,%d) value %g", e.code,
                  e.blk, e.i, e.j, e.value);
    return fail(map_dev_error(e.code), msg);
  }
  return AMR_OK;
}

// ------------------------------------------------------------- profiling
void Engine::prof_collect() {
  for (int q = 0; q + 1 < ev_used_; q += 2) {
    float ms = 0.f;
    if (cudaEventElapsedTime(&ms, ev_[q], ev_[q + 1]) == cudaSuccess) prof_.stage_ms += ms;
    else cudaGetLastError();  // a failed timing query must not surface in a later launch check
  }
  ev_used_ = 0;
  if (step_ev_pending_) {
    float ms = 0.f;
    if (cudaEventElapsedTime(&ms, step_ev_[0], step_ev_[1]) == cudaSuccess) prof_.step_gpu_ms += ms;
    else cudaGetLastError();
    step_ev_pending_ = false;
  }
  prof_.stage_cells += stage_cells_pending_;
  stage_cells_pending_ = 0;
}

int Engine::profile_enable(bool on) {
  if (stream_) CK(cudaStreamSynchronize(stream_), "sync");
  prof_ = amr_profile{};
  ev_used_ = 0;
  step_ev_pending_ = false;
  stage_cells_pending_ = 0;
  if (prof_on_ != on) gen_++;
  prof_on_ = on;
  return AMR_OK;
}

int Engine::profile_read(amr_profile *out) {
  if (!out) return fail(AMR_E_ARG, "null pointer");
  *out = prof_;
  return AMR_OK;
}

}  // namespace amr
