// Discrete adjoint of the frozen-mesh time step.  The forward step is
// recomputed from its checkpoint with a tape of the values the transposed
// kernels need, then the transposed step runs in reverse order of
// main.cpp:128-202.  No counterpart in the reference.
#include <cstring>

#include "adjoint_kernels.cuh"
#include "engine.hpp"
#include "stage_split.cuh"

namespace amr {

namespace {
constexpr int kNG = 2;  // the adjoint supports two ghost layers
using G2 = Geo<kNG>;

__global__ void k_scale(double *p, size_t n, double s) {
  const size_t i = static_cast<size_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i < n) p[i] *= s;
}

unsigned blocks_for(size_t n, unsigned b) { return static_cast<unsigned>((n + b - 1) / b); }
}  // namespace

#define CK(expr, where)                                 \
  do {                                                  \
    cudaError_t e_ = (expr);                            \
    if (e_ != cudaSuccess) return cuda_fail(e_, where); \
  } while (0)

int Engine::adjoint_supported() {
  if (f32_) return fail(AMR_E_UNSUPPORTED, "the adjoint runs on the FP64 path only");
  if (ng_ != kNG || m_.recon != REC_MUSCL || m_.flux != FLX_RUSA)
    return fail(AMR_E_UNSUPPORTED, "the adjoint covers MUSCL + RUSA with 2 ghost layers");
  for (const Instance &in : inst_) {
    if (in.limiter != LIM_MC && in.limiter != LIM_MINMOD)
      return fail(AMR_E_UNSUPPORTED, "the adjoint covers the MC and minmod limiters");
    if (in.cfg.maxlevs != 1) return fail(AMR_E_UNSUPPORTED, "the adjoint needs a frozen mesh (maxlevs 1)");
    if (!(in.cfg.dt_fixed > 0)) return fail(AMR_E_UNSUPPORTED, "the adjoint needs a fixed dt (dt_fixed > 0)");
    if (in.cfg.ct_type == 2 || in.cfg.diffusion)
      return fail(AMR_E_UNSUPPORTED, "the adjoint covers the basic CT EMF without diffusion");
  }
  return AMR_OK;
}

int Engine::adjoint_alloc() {
  const size_t cell = sizeof(double) * 8 * nn_ * cap_slots_, face = sizeof(double) * 2 * nn_ * cap_slots_;
  const size_t edge = sizeof(double) * nn_ * cap_slots_;
  for (DevBuf *b : {&a_U_, &a_Us_, &a_F_, &a_G_, &a_C_[0], &a_C_[1], &a_C_[2], &a_C_[3], &a_C_[4], &a_C_[5],
                    &a_C_[6], &a_C_[7], &t_W1_, &t_UsPre_, &t_UPre_}) {
    CK(b->ensure(cell), "adjoint alloc");
    CK(cudaMemsetAsync(b->p, 0, cell, stream_), "memset");
  }
  for (DevBuf *b : {&a_B_, &a_Bs_, &t_B1_, &t_BisF_, &t_BnewF_}) {
    CK(b->ensure(face), "adjoint alloc");
    CK(cudaMemsetAsync(b->p, 0, face, stream_), "memset");
  }
  CK(a_E_.ensure(edge), "adjoint alloc");
  CK(cudaMemsetAsync(a_E_.p, 0, edge, stream_), "memset");
  return AMR_OK;
}

int Engine::adjoint_enable(bool on) {
  if (on) {
    if (!initialised_) return fail(AMR_E_STATE, "amr_init has not been called");
    if (int rc = adjoint_supported()) return rc;
    if (int rc = adjoint_alloc()) return rc;
    CK(cudaStreamSynchronize(stream_), "sync");
  }
  adj_on_ = on;
  adj_gen_ = 0;  // the adjoint arrays may have moved: capture again
  ckpt_meta_.clear();
  for (DevBuf &b : ckpt_) b.release();
  ckpt_.clear();
  return AMR_OK;
}

// (U, Bi) of every used slot and the time-loop counters, before the step
int Engine::adjoint_record() {
  if (!ckpt_.empty() && static_cast<size_t>(used_slots_) != ckpt_slots_)
    return fail(AMR_E_STATE, "the block pool changed while recording the adjoint");
  ckpt_slots_ = static_cast<size_t>(used_slots_);
  const size_t u = sizeof(double) * 8 * nn_ * ckpt_slots_, b = sizeof(double) * 2 * nn_ * ckpt_slots_;
  DevBuf d;
  CK(d.ensure(u + b), "checkpoint alloc");
  ckpt_.push_back(d);
  CK(cudaMemcpyAsync(d.p, U_, u, cudaMemcpyDeviceToDevice, stream_), "checkpoint");
  CK(cudaMemcpyAsync(static_cast<char *>(d.p) + u, Bi_, b, cudaMemcpyDeviceToDevice, stream_), "checkpoint");
  Checkpoint c;
  for (const Instance &in : inst_) c.meta.push_back(InstMeta{in.t, in.dt, in.dtn, in.count, in.cell_updates});
  c.active = active_;
  ckpt_meta_.push_back(std::move(c));
  return AMR_OK;
}

int Engine::adjoint_seed(int q, int field, const double *lam, int64_t count) {
  if (!adj_on_) return fail(AMR_E_STATE, "the adjoint is not enabled");
  if (q < 0 || q >= static_cast<int>(inst_.size()) || !lam) return fail(AMR_E_ARG, "bad instance or pointer");
  if (field != AMR_FIELD_U && field != AMR_FIELD_BI) return fail(AMR_E_ARG, "adjoint fields are U and BI");
  const int f = field == AMR_FIELD_U ? kFieldAdjU : kFieldAdjB;
  Instance &in = inst_[q];
  if (count < static_cast<int64_t>(in.tree.lastActive) * field_nv(f) * nn_) return fail(AMR_E_ARG, "buffer too small");
  return xfer(in, f, const_cast<double *>(lam), true);
}

int Engine::adjoint_read(int q, int field, double *lam, int64_t count) {
  if (!adj_on_) return fail(AMR_E_STATE, "the adjoint is not enabled");
  if (q < 0 || q >= static_cast<int>(inst_.size()) || !lam) return fail(AMR_E_ARG, "bad instance or pointer");
  if (field != AMR_FIELD_U && field != AMR_FIELD_BI) return fail(AMR_E_ARG, "adjoint fields are U and BI");
  const int f = field == AMR_FIELD_U ? kFieldAdjU : kFieldAdjB;
  Instance &in = inst_[q];
  if (count < static_cast<int64_t>(in.tree.lastActive) * field_nv(f) * nn_) return fail(AMR_E_ARG, "buffer too small");
  return xfer(in, f, lam, false);
}

// CT2D with copies of the face field after its fill and of the cell state
// before the correction (the values k_ct_cell_adj needs)
int Engine::ct2d_taped(int step) {
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
  const size_t cell = sizeof(double) * 8 * nn_ * used_slots_, face = sizeof(double) * 2 * nn_ * used_slots_;
  CK(launch_ct_emf(m_, a, n, stream_), "ct emf");
  if (int rc = fill({{FILL_EC, AMR_FIELD_EMF}})) return rc;
  CK(launch_ct_face(m_, a, n, stream_), "ct face");
  if (int rc = fill({{FILL_FC, step == 1 ? AMR_FIELD_BIS : AMR_FIELD_BI}})) return rc;
  CK(cudaMemcpyAsync((step == 1 ? t_BisF_ : t_BnewF_).p, a.Bnew, face, cudaMemcpyDeviceToDevice, stream_), "tape");
  CK(cudaMemcpyAsync((step == 1 ? t_UsPre_ : t_UPre_).p, a.q, cell, cudaMemcpyDeviceToDevice, stream_), "tape");
  CK(launch_ct_cell(m_, a, n, stream_), "ct cell");
  prof_.launches += 3;
  return AMR_OK;
}

// main.cpp:129-202 from the restored checkpoint, keeping the tape
int Engine::adjoint_recompute() {
  const size_t cell = sizeof(double) * 8 * nn_ * used_slots_, face = sizeof(double) * 2 * nn_ * used_slots_;
  const bool split = split_;
  split_ = true;  // the tape needs the primitive state of each stage in W
  int rc = AMR_OK;
  cudaError_t e = cudaSuccess;
  do {
    if ((rc = fill({{FILL_CC, AMR_FIELD_U}, {FILL_FC, AMR_FIELD_BI}}))) break;
    if ((e = cudaMemcpyAsync(t_B1_.p, Bi_, face, cudaMemcpyDeviceToDevice, stream_)) != cudaSuccess) break;
    if ((rc = stage(1))) break;
    if ((e = cudaMemcpyAsync(t_W1_.p, W_, cell, cudaMemcpyDeviceToDevice, stream_)) != cudaSuccess) break;
    if ((rc = fill({{FILL_FC, AMR_FIELD_BI}, {FILL_FC, AMR_FIELD_FF}, {FILL_FC, AMR_FIELD_GG}}))) break;
    if ((rc = ct2d_taped(1))) break;
    if ((rc = fill({{FILL_CC, AMR_FIELD_US}}))) break;
    if ((rc = stage(2))) break;  // leaves the stage-2 primitive state in W
    if ((rc = fill({{FILL_FC, AMR_FIELD_FF}, {FILL_FC, AMR_FIELD_GG}}))) break;
    if ((rc = ct2d_taped(2))) break;
    rc = fill({{FILL_CC, AMR_FIELD_U}});
  } while (false);
  split_ = split;
  if (e != cudaSuccess) return cuda_fail(e, "tape");
  return rc;
}

// transpose of one compiled fill, on up to three adjoint arrays
int Engine::ghost_adj(std::initializer_list<AdjSeg> what) {
  if (nops_ == 0) return AMR_OK;
  GhostAdjLaunch g{};
  g.ops = d_ops_.as<GhostOp>();
  g.snaps = d_snaps_.as<GhostSnap>();
  g.nops = static_cast<int>(nops_);
  int q = 0;
  for (const AdjSeg &w : what) {
    GhostSeg &s = g.seg[q++];
    s.field = w.a;
    s.kind = w.kind;
    s.nv = w.nv;
    s.f32 = 0;
  }
  g.nseg = q;
  g.take = a_take_.as<double>();  // sized by adjoint_step
  const size_t n = static_cast<size_t>(g.nops) * g.nseg;
  k_ghost_adj_take<G2::N><<<blocks_for(n, 256), 256, 0, stream_>>>(g);
  k_ghost_adj_give<G2::N><<<blocks_for(n, 256), 256, 0, stream_>>>(g);
  CK(cudaGetLastError(), "ghost adjoint");
  prof_.launches += 2;
  return AMR_OK;
}

// the transposed step (the adjoint of the state after the step is in aU, aB)
int Engine::adjoint_sequence() {
  const int nt = static_cast<int>(tasks_.size());
  const size_t cell = sizeof(double) * 8 * nn_ * used_slots_, face = sizeof(double) * 2 * nn_ * used_slots_;
  const size_t edge = sizeof(double) * nn_ * used_slots_;
  double *aU = a_U_.as<double>(), *aUs = a_Us_.as<double>(), *aB = a_B_.as<double>(), *aBs = a_Bs_.as<double>();
  double *aE = a_E_.as<double>(), *aF = a_F_.as<double>(), *aG = a_G_.as<double>();
  for (void *p : {static_cast<void *>(aUs), static_cast<void *>(aF), static_cast<void *>(aG)})
    CK(cudaMemsetAsync(p, 0, cell, stream_), "memset");
  CK(cudaMemsetAsync(aBs, 0, face, stream_), "memset");
  CK(cudaMemsetAsync(aE, 0, edge, stream_), "memset");

  auto ct_args = [&](int step) {
    CtAdjArgs c{};
    c.tasks = d_tasks_.as<LeafTask>();
    c.inst = d_params_.as<InstParams>();
    c.step = step;
    c.Bnew = step == 1 ? t_BisF_.as<double>() : t_BnewF_.as<double>();
    c.qpre = step == 1 ? t_UsPre_.as<double>() : t_UPre_.as<double>();
    c.aq = step == 1 ? aUs : aU;
    c.aBnew = step == 1 ? aBs : aB;
    c.aBsrc = step == 1 ? aB : aBs;
    c.aE = aE;
    c.aF = aF;
    c.aG = aG;
    return c;
  };
  auto st_args = [&](int step) {
    StageAdjArgs s{};
    s.tasks = d_tasks_.as<LeafTask>();
    s.inst = d_params_.as<InstParams>();
    s.step = step;
    s.ntasks = nt;
    s.W = step == 1 ? t_W1_.as<double>() : static_cast<const double *>(W_);
    s.B = step == 1 ? t_B1_.as<double>() : t_BisF_.as<double>();
    s.aOut = step == 1 ? aUs : aU;
    s.aIn = step == 1 ? aU : aUs;
    s.aF = aF;
    s.aG = aG;
    s.aB = step == 1 ? aB : aBs;
    for (int d = 0; d < 2; d++)
      for (int q = 0; q < 4; q++) s.C[d][q] = a_C_[4 * d + q].as<double>();
    return s;
  };
  const size_t nface = static_cast<size_t>(nt) * 2 * G2::NF * G2::NF;
  const size_t ncell = static_cast<size_t>(nt) * G2::NN;
  int rc;
  for (int step = 2; step >= 1; step--) {
    // fill of the stage output (U after stage 2, Us after stage 1)
    if ((rc = ghost_adj({{FILL_CC, step == 2 ? aU : aUs, 8}}))) return rc;
    const CtAdjArgs c = ct_args(step);
    k_ct_cell_adj<kNG><<<nt, 128, 0, stream_>>>(c);
    if ((rc = ghost_adj({{FILL_FC, c.aBnew, 2}}))) return rc;
    k_ct_face_adj<kNG><<<nt, 128, 0, stream_>>>(c);
    if (step == 2) {
      k_scale<<<blocks_for(face / sizeof(double), 256), 256, 0, stream_>>>(aB, face / sizeof(double), 0.5);
    } else {
      CK(cudaMemsetAsync(aBs, 0, face, stream_), "memset");
    }
    if ((rc = ghost_adj({{FILL_EC, aE, 1}}))) return rc;
    k_ct_emf_adj<kNG><<<nt, 128, 0, stream_>>>(c);
    CK(cudaMemsetAsync(aE, 0, edge, stream_), "memset");
    if (step == 2) {
      if ((rc = ghost_adj({{FILL_FC, aF, 8}, {FILL_FC, aG, 8}}))) return rc;
    } else {
      if ((rc = ghost_adj({{FILL_FC, aB, 2}, {FILL_FC, aF, 8}, {FILL_FC, aG, 8}}))) return rc;
    }
    const StageAdjArgs s = st_args(step);
    k_faces_adj<kNG><<<blocks_for(nface, 128), 128, 0, stream_>>>(s);
    k_cells_adj<kNG><<<blocks_for(ncell, 256), 256, 0, stream_>>>(s);
    CK(cudaGetLastError(), "adjoint kernels");
    prof_.launches += 6;
    CK(cudaMemsetAsync(aF, 0, cell, stream_), "memset");
    CK(cudaMemsetAsync(aG, 0, cell, stream_), "memset");
  }
  // the first fills of the step (U and Bi)
  return ghost_adj({{FILL_CC, aU, 8}, {FILL_FC, aB, 2}});
}

int Engine::adjoint_enqueue() {
  if (int rc = adjoint_recompute()) return rc;
  return adjoint_sequence();
}

// One step back: restore the last checkpoint, recompute that step with its
// tape, apply the transposed step, and leave the state at the checkpoint.
int Engine::adjoint_step() {
  if (!adj_on_) return fail(AMR_E_STATE, "the adjoint is not enabled");
  if (poisoned_) return fail(AMR_E_STATE, "engine stopped by an earlier error: " + last_error);
  if (ckpt_meta_.empty()) return fail(AMR_E_STATE, "no recorded step left to reverse");
  if (a_U_.bytes < sizeof(double) * 8 * nn_ * static_cast<size_t>(cap_slots_))
    return fail(AMR_E_STATE, "the block pool changed since the adjoint was enabled");
  const Checkpoint &c = ckpt_meta_.back();
  DevBuf &d = ckpt_.back();
  const size_t u = sizeof(double) * 8 * nn_ * ckpt_slots_, b = sizeof(double) * 2 * nn_ * ckpt_slots_;
  active_ = c.active;
  if (int rc = rebuild()) return rc;
  for (size_t q = 0; q < inst_.size(); q++) {
    inst_[q].dt = c.meta[q].dt;
    inst_[q].dtn = c.meta[q].dtn;
  }
  if (int rc = upload_params()) return rc;
  CK(a_take_.ensure(sizeof(double) * 16 * kMaxSeg * static_cast<size_t>(nops_ > 0 ? nops_ : 1)), "alloc");
  CK(cudaMemcpyAsync(U_, d.p, u, cudaMemcpyDeviceToDevice, stream_), "restore");
  CK(cudaMemcpyAsync(Bi_, static_cast<char *>(d.p) + u, b, cudaMemcpyDeviceToDevice, stream_), "restore");
  if (!graph_on_ || prof_on_) {
    if (int rc = adjoint_enqueue()) return rc;
  } else {
    if (!adj_exec_ || adj_gen_ != gen_) {  // capture once per tree and pool
      if (adj_exec_) { cudaGraphExecDestroy(adj_exec_); adj_exec_ = nullptr; }
      cudaStream_t user = stream_;
      stream_ = cap_stream_;
      cudaError_t e = cudaStreamBeginCapture(cap_stream_, cudaStreamCaptureModeRelaxed);
      if (e != cudaSuccess) { stream_ = user; return cuda_fail(e, "graph capture"); }
      capturing_ = true;
      int rc = adjoint_enqueue();
      capturing_ = false;
      cudaGraph_t g = nullptr;
      e = cudaStreamEndCapture(cap_stream_, &g);
      stream_ = user;
      if (rc) { if (g) cudaGraphDestroy(g); return rc; }
      if (e != cudaSuccess) return cuda_fail(e, "graph capture");
      e = cudaGraphInstantiate(&adj_exec_, g, 0);
      cudaGraphDestroy(g);
      if (e != cudaSuccess) { adj_exec_ = nullptr; return cuda_fail(e, "graph instantiate"); }
      adj_gen_ = gen_;
    }
    CK(cudaGraphLaunch(adj_exec_, stream_), "graph launch");
  }
  CK(cudaMemcpyAsync(U_, d.p, u, cudaMemcpyDeviceToDevice, stream_), "restore");
  CK(cudaMemcpyAsync(Bi_, static_cast<char *>(d.p) + u, b, cudaMemcpyDeviceToDevice, stream_), "restore");
  if (int rc = check_device_error()) return rc;
  for (size_t q = 0; q < inst_.size(); q++) {
    Instance &in = inst_[q];
    const InstMeta &m = c.meta[q];
    in.t = m.t;
    in.dt = m.dt;
    in.dtn = m.dtn;
    in.count = m.count;
    in.cell_updates = m.cell_updates;
    in.done = false;
  }
  d.release();
  ckpt_.pop_back();
  ckpt_meta_.pop_back();
  return AMR_OK;
}

}  // namespace amr
