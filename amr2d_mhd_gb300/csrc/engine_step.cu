// Engine: initialisation, the time step, remeshing and the reference-function
// entry points.
#include <chrono>
#include <cmath>
#include <cstring>

#include "aux_kernels.cuh"
#include "engine.hpp"
#include "host_par.hpp"

namespace amr {

#define CK(expr, where)                                 \
  do {                                                  \
    cudaError_t e_ = (expr);                            \
    if (e_ != cudaSuccess) return cuda_fail(e_, where); \
  } while (0)

// copy blocks [0, lastActive) of one field between a dense float64 host
// array [block][var][j][i] and the slot pool.  From or into page-locked
// memory the scatter / gather kernel reads or writes the caller's array
// directly: one pass over the link and no staging copy (2.6 % more
// end-to-end cell-updates/s on the rotor; for pageable memory the kernel's
// accesses through the host page tables were 5 % slower than the copy, so
// pageable arrays keep it).  Otherwise the bulk copy goes between the caller's array and
// a device staging buffer (the driver's pageable path, direct DMA on a
// coherent link, beats a host memcpy into pinned memory followed by a pinned
// copy) and the kernel moves the blocks between the staging buffer and their
// slots.  A pageable host-to-device copy has read its source when it
// returns, so that upload returns without waiting for the device (later work
// on the stream is ordered after the scatter); every other upload, and every
// download, waits, so that the caller may reuse or read the array at once.
int Engine::xfer(Instance &in, int field, double *host, bool to_device) {
  const int nblk = in.tree.lastActive;
  const int per = field_nv(field) * nn_;
  const size_t bytes = static_cast<size_t>(nblk) * per * sizeof(double);
  if (nblk == 0) return AMR_OK;
  if (nblk > in.slotmap_n) {  // slots are never reassigned: only new blocks need uploading
    if (sizeof(int) * nblk > in.d_slotmap.bytes) CK(cudaStreamSynchronize(stream_), "sync");
    CK(in.d_slotmap.ensure(sizeof(int) * nblk), "alloc");
    // a pageable source: read by the time the call returns
    CK(cudaMemcpyAsync(in.d_slotmap.p, in.slot.data(), sizeof(int) * nblk, cudaMemcpyHostToDevice, stream_), "h2d");
    prof_.h2d_bytes += static_cast<int64_t>(sizeof(int) * nblk);
    in.slotmap_n = nblk;
  }
  const int *slots = in.d_slotmap.as<int>();
  void *fp = field_ptr(field);
  // the device's view of the caller's array, if it has one
  double *direct = nullptr;
  bool pinned = false;
  {
    cudaPointerAttributes pa{};
    if (cudaPointerGetAttributes(&pa, host) != cudaSuccess) {
      cudaGetLastError();  // an unknown (pageable) pointer on older runtimes
    } else if (pa.type == cudaMemoryTypeHost || pa.type == cudaMemoryTypeManaged) {
      pinned = true;
      if (zero_copy_ && pa.type == cudaMemoryTypeHost && pa.devicePointer)
        direct = static_cast<double *>(pa.devicePointer);
    }
  }
  if (direct) {
    if (to_device) {
      CK(launch_scatter(slots, nblk, fp, field_f32(field), per, direct, stream_), "scatter");
      prof_.h2d_bytes += static_cast<int64_t>(bytes);
    } else {
      CK(launch_gather(slots, nblk, fp, field_f32(field), per, direct, stream_), "gather");
      prof_.d2h_bytes += static_cast<int64_t>(bytes);
    }
    prof_.launches += 1;
    CK(cudaStreamSynchronize(stream_), "sync");
    return AMR_OK;
  }
  // a growing staging buffer is freed and reallocated: let an earlier
  // upload's scatter finish reading it first
  if (bytes > d_stage_.bytes) CK(cudaStreamSynchronize(stream_), "sync");
  CK(d_stage_.ensure(bytes), "alloc");
  if (to_device) {
    CK(cudaMemcpyAsync(d_stage_.p, host, bytes, cudaMemcpyHostToDevice, stream_), "h2d");
    CK(launch_scatter(slots, nblk, fp, field_f32(field), per, d_stage_.as<double>(), stream_), "scatter");
    prof_.h2d_bytes += static_cast<int64_t>(bytes);
    prof_.launches += 1;
    if (pinned) CK(cudaStreamSynchronize(stream_), "sync");
  } else {
    CK(launch_gather(slots, nblk, fp, field_f32(field), per, d_stage_.as<double>(), stream_), "gather");
    prof_.d2h_bytes += static_cast<int64_t>(bytes);
    prof_.launches += 1;
    CK(cudaMemcpyAsync(host, d_stage_.p, bytes, cudaMemcpyDeviceToHost, stream_), "d2h");
    CK(cudaStreamSynchronize(stream_), "sync");
  }
  return AMR_OK;
}

// admesh.cpp:17-102 for the instances in `which`; the criterion comes from the
// device reduction of the last dt_crit (or, at initialisation, from k_ic's),
// or the caller's marks replace it (`marks`, one instance).  The refine / coarsen kernels run while the
// host compiles the changed instances' ghost programs; the device error check
// (U2W("refine") traps) follows, so errors surface before the call returns.
int Engine::admesh_all(const std::vector<int> &which, const std::vector<std::vector<double>> *host_grad,
                       const AdmeshMarks *marks) {
  const auto t0 = std::chrono::steady_clock::now();
  std::vector<TreeOp> ref, crs;
  // the quadtrees of a batch are independent: admesh them on host threads,
  // then give the new blocks slots in instance order (the pool may grow)
  std::vector<AdmeshPlan> plans(which.size());
  std::vector<std::string> errs(which.size());
  std::vector<char> ok(which.size(), 1);
  size_t blocks = 0;
  for (int q : which) blocks += static_cast<size_t>(inst_[q].tree.lastActive);
  parallel_items(pool_, which.size(), host_threads(blocks), [&](size_t, size_t w) {
    Instance &in = inst_[which[w]];
    if (in.cfg.maxlevs <= 1) return;
    if (marks) {
      ok[w] = in.tree.admesh_marked(marks->ref, marks->crs, plans[w], errs[w]) ? 1 : 0;
      return;
    }
    std::vector<double> grad(in.tree.lastActive, 0.0);
    if (host_grad) {
      grad = (*host_grad)[which[w]];
    } else {
      const double *hg = h_grad_.as<double>();
      for (int t = in.task_begin; t < in.task_end; t++) grad[task_blk_[t]] = hg[t];
    }
    ok[w] = in.tree.admesh(grad, plans[w], errs[w]) ? 1 : 0;
  });
  for (size_t w = 0; w < which.size(); w++) {
    const int q = which[w];
    Instance &in = inst_[q];
    if (in.cfg.maxlevs <= 1) continue;
    if (!ok[w]) return fail(AMR_E_MAXBLOCKS, errs[w]);
    if (int rc = assign_slots(in)) return rc;
    const AdmeshPlan &plan = plans[w];
    for (const auto &r : plan.refine)
      ref.push_back(TreeOp{in.slot[r[0]], {in.slot[r[1]], in.slot[r[2]], in.slot[r[3]], in.slot[r[4]]}, q});
    for (const auto &c : plan.coarsen)
      crs.push_back(TreeOp{in.slot[c[0]], {in.slot[c[1]], in.slot[c[2]], in.slot[c[3]], in.slot[c[4]]}, q});
  }
  prof_.host_admesh_ms += std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
  if (ref.empty() && crs.empty()) return AMR_OK;
  if (int rc = upload_params()) return rc;
  std::vector<TreeOp> all(ref);
  all.insert(all.end(), crs.begin(), crs.end());
  CK(d_treeops_.ensure(sizeof(TreeOp) * all.size()), "alloc");
  CK(cudaMemcpyAsync(d_treeops_.p, all.data(), sizeof(TreeOp) * all.size(), cudaMemcpyHostToDevice, stream_),
     "h2d");
  TreeOpArgs a{};
  a.ops = d_treeops_.as<TreeOp>();
  a.inst = d_params_.as<InstParams>();
  a.U = U_;
  a.Bi = Bi_;
  a.err = d_err_.as<DevError>();
  CK(launch_refine(m_, a, static_cast<int>(ref.size()), stream_), "refine");
  a.ops = d_treeops_.as<TreeOp>() + ref.size();
  CK(launch_coarsen(m_, a, static_cast<int>(crs.size()), stream_), "coarsen");
  prof_.launches += (ref.empty() ? 0 : 1) + (crs.empty() ? 0 : 1);
  prof_.h2d_bytes += static_cast<int64_t>(sizeof(TreeOp) * all.size());
  if (initialised_) {
    const auto t1 = std::chrono::steady_clock::now();
    if (int rc = compile_programs()) return rc;
    prof_.host_compile_ms += std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t1).count();
  }
  return check_device_error();  // also keeps `all` alive until the copy is done
}

// basegrid + IC2Dtype + W2U + initial admesh (main.cpp:97-116).  The root
// blocks' initial condition, face field and criterion come from k_ic (one
// launch over the roots of every instance); the host prepares each block's
// constants and 1-D profiles (ic_prepare) and runs the initial admesh on the
// criterion.
int Engine::init() {
  if (initialised_) return fail(AMR_E_STATE, "amr_init called twice");
  if (poisoned_) return fail(AMR_E_STATE, "engine stopped by an earlier error");
  std::vector<IcDev> blocks;
  std::vector<double> tabs;
  std::vector<std::pair<int, int>> owner;   // (instance, block ID) of each root block
  for (size_t q = 0; q < inst_.size(); q++) {
    Instance &in = inst_[q];
    in.tree.basegrid();
    if (int rc = assign_slots(in)) return rc;
    for (int nb = 0; nb < in.tree.lastActive; nb++) {
      IcBlock b{n_, ng_, in.tree.icoord[nb][0], in.tree.icoord[nb][1], in.dx[0], in.dy[0],
                in.cfg.geometry == 0 ? in.dx[0] : 0.0, in.cfg.geometry == 0 ? in.dy[0] : 0.0};
      IcDev d;
      std::vector<double> t(static_cast<size_t>(3) * n_);
      if (ic_prepare(in.ic, in.cfg.ic_param, b, in.gamma, d, t.data())) {
        d.tab = static_cast<int>(tabs.size() / n_);
        tabs.insert(tabs.end(), t.begin(), t.end());
      }
      d.slot = in.slot[nb];
      blocks.push_back(d);
      owner.emplace_back(static_cast<int>(q), nb);
    }
    in.t = 0.0;
    in.dt = 0.0;  // dom.dt is read before its first assignment (main.cpp:154 vs :231)
    in.dtn = 0.0;
    if (in.cfg.dt_fixed > 0) in.dt = in.dtn = in.cfg.dt_fixed;
    in.count = 0;
  }
  const size_t nb = blocks.size();
  if (tabs.empty()) tabs.assign(1, 0.0);
  DevBuf d_blocks, d_tabs;
  CK(d_blocks.ensure(sizeof(IcDev) * nb), "alloc");
  CK(d_tabs.ensure(sizeof(double) * tabs.size()), "alloc");
  CK(d_grad_.ensure(sizeof(double) * nb), "alloc");
  CK(h_grad_.ensure(sizeof(double) * nb), "alloc");
  CK(cudaMemcpyAsync(d_blocks.p, blocks.data(), sizeof(IcDev) * nb, cudaMemcpyHostToDevice, stream_), "h2d");
  CK(cudaMemcpyAsync(d_tabs.p, tabs.data(), sizeof(double) * tabs.size(), cudaMemcpyHostToDevice, stream_), "h2d");
  CK(launch_ic(m_, d_blocks.as<IcDev>(), static_cast<int>(nb), d_tabs.as<double>(), U_, Bi_, d_grad_.as<double>(),
               stream_), "initial condition");
  CK(cudaMemcpyAsync(h_grad_.p, d_grad_.p, sizeof(double) * nb, cudaMemcpyDeviceToHost, stream_), "d2h");
  CK(cudaStreamSynchronize(stream_), "sync");  // also keeps the host arrays alive until the copies ran
  prof_.launches += 1;
  prof_.h2d_bytes += static_cast<int64_t>(sizeof(IcDev) * nb + sizeof(double) * tabs.size());
  prof_.d2h_bytes += static_cast<int64_t>(sizeof(double) * nb);
  d_blocks.release();
  d_tabs.release();
  std::vector<std::vector<double>> grads(inst_.size());
  for (size_t q = 0; q < inst_.size(); q++) grads[q].assign(inst_[q].tree.lastActive, 0.0);
  for (size_t k = 0; k < nb; k++) grads[owner[k].first][owner[k].second] = h_grad_.as<double>()[k];
  std::vector<int> all(inst_.size());
  for (size_t q = 0; q < inst_.size(); q++) all[q] = static_cast<int>(q);
  if (int rc = admesh_all(all, &grads)) return rc;
  initialised_ = true;
  return AMR_OK;
}

int Engine::finish_step() {
  const size_t nt = tasks_.size();
  prof_.d2h_bytes += static_cast<int64_t>(2 * sizeof(double) * nt);
  prof_.steps += 1;
  if (int rc = check_device_error()) return rc;
  const double *hl = h_lambda_.as<double>();
  for (int a : active_) {
    Instance &in = inst_[a];
    double lambda = 1.E6;  // main.cpp:209, 228
    for (int t = in.task_begin; t < in.task_end; t++) {
      const double v = (tasks_[t].dx < tasks_[t].dy ? tasks_[t].dx : tasks_[t].dy) / hl[t];
      lambda = v < lambda ? v : lambda;
    }
    in.count = in.count + 1;
    in.cell_updates += static_cast<int64_t>(in.task_end - in.task_begin) * NI * NI;
    if (in.cfg.dt_fixed > 0) {  // fixed step: t advances by the dt this step used
      in.t = in.t + in.cfg.dt_fixed;
      continue;
    }
    in.t = in.t + in.dtn;  // main.cpp:231-234
    in.dt = in.dtn;
    in.dtn = in.cfl * lambda;
    if (in.dtn < 0 || std::isnan(in.dtn)) return fail(AMR_E_DT, "invalid dt produced");
  }
  if (!remesh_) return AMR_OK;
  return admesh_all(active_, nullptr);
}

// one iteration of main.cpp:128-247 for every instance with t <= t_end
int Engine::step() {
  if (int rc = step_begin()) return rc;
  return step_end();
}

// the device half of a step: leaf list and ghost programs of the current
// trees, then the step's launches; returns without waiting for the device
int Engine::step_begin() {
  if (!initialised_) return fail(AMR_E_STATE, "amr_init has not been called");
  if (poisoned_) return fail(AMR_E_STATE, "engine stopped by an earlier error: " + last_error);
  if (step_pending_) return fail(AMR_E_STATE, "a step is already in flight");
  active_.clear();
  for (size_t q = 0; q < inst_.size(); q++) {
    Instance &in = inst_[q];
    if (!in.done && !(in.t <= in.t_end)) in.done = true;
    if (!in.done) active_.push_back(static_cast<int>(q));
  }
  if (active_.empty()) return AMR_OK;
  if (int rc = rebuild()) return rc;
  if (adj_on_)
    if (int rc = adjoint_record()) return rc;
  if (int rc = launch_step()) return rc;
  step_pending_ = true;
  return AMR_OK;
}

// the host half: wait for the step, advance t / dt, remesh (and compile the
// changed trees' ghost programs while the refine / coarsen kernels run)
int Engine::step_end() {
  if (!step_pending_) return AMR_OK;
  step_pending_ = false;
  return finish_step();
}

int Engine::run(int64_t max_steps) {
  for (int64_t s = 0; max_steps < 0 || s < max_steps; s++) {
    bool any = false;
    for (const Instance &in : inst_) any |= !in.done && in.t <= in.t_end;
    if (!any) break;
    if (int rc = step()) return rc;
  }
  return AMR_OK;
}

int Engine::info(int q, amr_info *o) {
  if (q < 0 || q >= static_cast<int>(inst_.size()) || !o) return fail(AMR_E_ARG, "bad instance or pointer");
  const Instance &in = inst_[q];
  std::memset(o, 0, sizeof(*o));
  o->t = in.t;
  o->dt = in.dt;
  o->dt_next = in.dtn;
  o->t_end = in.t_end;
  o->gamma = in.gamma;
  o->steps = in.count;
  o->last_active = in.tree.lastActive;
  int nl = 0;
  for (int b = 0; b < in.tree.lastActive; b++) nl += in.tree.leafs[b];
  o->n_leaves = nl;
  o->nb_leafs = in.tree.nbleafs;
  o->done = (in.done || !(in.t <= in.t_end)) ? 1 : 0;
  o->n_instances = static_cast<int>(inst_.size());
  o->nx_tot = n_;
  o->ny_tot = n_;
  o->cell_updates = in.cell_updates;
  return AMR_OK;
}

// ------------------------------------------------ reference-function level
int Engine::api_locate_bounds() {
  if (!initialised_) return fail(AMR_E_STATE, "amr_init has not been called");
  active_ = {0};
  programs_valid_ = false;
  return rebuild();
}

int Engine::api_boundary(int field) {
  if (int rc = api_locate_bounds()) return rc;
  FillKind k;
  if (field == AMR_FIELD_U || field == AMR_FIELD_US) k = FILL_CC;
  else if (field == AMR_FIELD_EMF) k = FILL_EC;
  else if (field == AMR_FIELD_BI || field == AMR_FIELD_BIS || field == AMR_FIELD_FF || field == AMR_FIELD_GG) k = FILL_FC;
  else return fail(AMR_E_ARG, "no ghost fill for this field");
  if (int rc = fill({{k, field}})) return rc;
  return check_device_error();
}

int Engine::api_muscl2d_rk(int step) {
  if (step != 1 && step != 2) return fail(AMR_E_ARG, "step must be 1 or 2");
  if (int rc = api_locate_bounds()) return rc;
  if (int rc = upload_params()) return rc;
  if (int rc = stage(step)) return rc;
  return check_device_error();
}

int Engine::api_ct2d(int step) {
  if (step != 1 && step != 2) return fail(AMR_E_ARG, "step must be 1 or 2");
  if (int rc = api_locate_bounds()) return rc;
  if (int rc = upload_params()) return rc;
  if (int rc = ct2d(step)) return rc;
  return check_device_error();
}

int Engine::api_cfl_dt(double *lambda_min) {
  if (!lambda_min) return fail(AMR_E_ARG, "null pointer");
  if (int rc = api_locate_bounds()) return rc;
  if (int rc = upload_params()) return rc;
  if (int rc = dt_crit(true)) return rc;
  const size_t nt = tasks_.size();
  CK(cudaMemcpyAsync(h_lambda_.p, d_lambda_.p, sizeof(double) * nt, cudaMemcpyDeviceToHost, stream_), "d2h");
  CK(cudaMemcpyAsync(h_grad_.p, d_grad_.p, sizeof(double) * nt, cudaMemcpyDeviceToHost, stream_), "d2h");
  if (int rc = check_device_error()) return rc;
  double lambda = 1.E6;
  for (size_t t = 0; t < nt; t++) {
    const double v = (tasks_[t].dx < tasks_[t].dy ? tasks_[t].dx : tasks_[t].dy) / h_lambda_.as<double>()[t];
    lambda = v < lambda ? v : lambda;
  }
  *lambda_min = lambda;
  return AMR_OK;
}

// criteria.cpp:6-44 on the current state: per block ID of instance 0 the
// largest relative jump of p, rho, Bx, By over its interior cells (leaves;
// -1 for blocks that are not leaves), from the same device reduction the
// step uses
int Engine::api_criteria(double *grad, int32_t cap) {
  if (!grad) return fail(AMR_E_ARG, "null pointer");
  double lam;
  if (int rc = api_cfl_dt(&lam)) return rc;
  const Instance &in = inst_[0];
  if (cap < in.tree.lastActive) return fail(AMR_E_ARG, "buffer too small");
  for (int b = 0; b < in.tree.lastActive; b++) grad[b] = -1.0;
  const double *hg = h_grad_.as<double>();
  for (int t = in.task_begin; t < in.task_end; t++) grad[task_blk_[t]] = hg[t];
  return AMR_OK;
}

// criteria.cpp:31,43 (markref.cpp:6-18) on the device criterion of each leaf
int Engine::api_criteria_flags(uint8_t *iref, uint8_t *icoarse, int32_t cap) {
  if (!iref || !icoarse) return fail(AMR_E_ARG, "null pointer");
  const Instance &in = inst_[0];
  std::vector<double> g(static_cast<size_t>(in.tree.lastActive > 0 ? in.tree.lastActive : 1));
  if (cap < in.tree.lastActive) return fail(AMR_E_ARG, "buffer too small");
  if (int rc = api_criteria(g.data(), static_cast<int32_t>(g.size()))) return rc;
  for (int b = 0; b < in.tree.lastActive; b++) {
    iref[b] = 0;
    icoarse[b] = 0;
    if (!in.tree.leafs[b]) continue;
    if (g[b] >= 0.05) {
      if (in.tree.lp[b][0] < in.cfg.maxlevs - 1) iref[b] = 1;
    } else if (g[b] <= 1.0) {
      icoarse[b] = 1;
    }
  }
  return AMR_OK;
}

// admesh.cpp:17-102 on instance 0 with the caller's refine / coarsen marks
// (per block ID) in place of criteria.cpp's
int Engine::api_admesh_marked(const uint8_t *iref, const uint8_t *icoarse, int32_t n) {
  if (!initialised_) return fail(AMR_E_STATE, "amr_init has not been called");
  if (!iref || !icoarse) return fail(AMR_E_ARG, "null pointer");
  if (n < inst_[0].tree.lastActive) return fail(AMR_E_ARG, "fewer marks than last_active blocks");
  const AdmeshMarks m{iref, icoarse};
  return admesh_all({0}, nullptr, &m);
}

int Engine::api_admesh() {
  double lam;
  if (int rc = api_cfl_dt(&lam)) return rc;
  return admesh_all({0}, nullptr);
}

// ------------------------------------------------------------ state exchange
int Engine::get_tree(int q, int32_t *lp, int32_t *icoord, uint8_t *leafs, int32_t cap) {
  if (q < 0 || q >= static_cast<int>(inst_.size())) return fail(AMR_E_ARG, "bad instance");
  const Tree &t = inst_[q].tree;
  if (cap < t.lastActive) return fail(AMR_E_ARG, "capacity smaller than last_active");
  for (int b = 0; b < t.lastActive; b++) {
    if (lp) std::memcpy(lp + 8 * b, t.lp[b].data(), 8 * sizeof(int32_t));
    if (icoord) { icoord[2 * b] = t.icoord[b][0]; icoord[2 * b + 1] = t.icoord[b][1]; }
    if (leafs) leafs[b] = t.leafs[b];
  }
  return AMR_OK;
}

int Engine::download(int q, int field, double *dst, int64_t count) {
  if (q < 0 || q >= static_cast<int>(inst_.size()) || !dst) return fail(AMR_E_ARG, "bad instance or pointer");
  Instance &in = inst_[q];
  const bool w = field == AMR_FIELD_W;
  const int f = w ? AMR_FIELD_U : field;
  if (!field_ptr(f)) return fail(AMR_E_ARG, "unknown field");
  const int64_t need = static_cast<int64_t>(in.tree.lastActive) * field_nv(f) * nn_;
  if (count < need) return fail(AMR_E_ARG, "buffer too small");
  if (int rc = xfer(in, f, dst, false)) return rc;
  if (w) {  // meshblock.cpp:119-145 on the host
    const double g = in.gamma;
    for (int b = 0; b < in.tree.lastActive; b++) {
      double *u = dst + static_cast<size_t>(b) * 8 * nn_;
      for (int c = 0; c < nn_; c++) {
        double x[8];
        for (int k = 0; k < 8; k++) x[k] = u[k * nn_ + c];
        const double w1 = x[1] / x[0], w2 = x[2] / x[0], w3 = x[3] / x[0];
        double p = (g - 1) * (x[4] - 0.5 * x[0] * (w1 * w1 + w2 * w2 + w3 * w3));
        p = p - (g - 1) * (0.5 * (x[5] * x[5] + x[6] * x[6] + x[7] * x[7]));
        u[1 * nn_ + c] = w1; u[2 * nn_ + c] = w2; u[3 * nn_ + c] = w3; u[4 * nn_ + c] = p;
      }
    }
  }
  return AMR_OK;
}

// the quadtree and time state of a run the caller owns (amr_set_tree); the
// handle counts as initialised once every instance has one
int Engine::api_set_tree(int q, int32_t na, int32_t nbl, const int32_t *lp, const int32_t *icoord,
                         const uint8_t *leafs, double t, double dt, double dtn, int64_t steps) {
  if (initialised_) return fail(AMR_E_STATE, "amr_set_tree takes the place of amr_init");
  if (q < 0 || q >= static_cast<int>(inst_.size()) || !lp || !icoord || !leafs)
    return fail(AMR_E_ARG, "bad instance or pointer");
  Instance &in = inst_[q];
  if (na < 1 || na > in.tree.maxblocks()) return fail(AMR_E_MAXBLOCKS, "last_active outside [1, maxblocks]");
  // built in a fresh tree (IDs from na on as a new tree has them) and checked
  // before it replaces the instance's: its IDs index slots, ghost programs
  // and refine / coarsen operations
  Tree tr(in.tree.shape());
  for (int b = 0; b < na; b++) {
    for (int k = 0; k < 8; k++) tr.lp[b][k] = lp[8 * b + k];
    tr.icoord[b] = {icoord[2 * b], icoord[2 * b + 1]};
    tr.leafs[b] = leafs[b] ? 1 : 0;
    if (tr.lp[b][0] < 0 || tr.lp[b][0] >= in.cfg.maxlevs) return fail(AMR_E_CONFIG, "block level outside maxlevs");
  }
  tr.lastActive = na;
  std::string err;
  if (!tr.check(err)) return fail(AMR_E_ARG, "amr_set_tree: " + err);
  tr.nbleafs = nbl;
  tr.version = in.tree.version + 1;
  in.tree = std::move(tr);
  in.t = t;
  in.dt = dt;
  in.dtn = dtn;
  in.count = steps;
  in.cell_updates = 0;
  in.done = false;
  if (int rc = assign_slots(in)) return rc;
  in.handed = true;
  bool all = true;
  for (const Instance &x : inst_) all = all && x.handed;
  if (all) {
    programs_valid_ = false;
    initialised_ = true;
  }
  return AMR_OK;
}

int Engine::upload(int q, int field, const double *src, int64_t count) {
  if (q < 0 || q >= static_cast<int>(inst_.size()) || !src) return fail(AMR_E_ARG, "bad instance or pointer");
  Instance &in = inst_[q];
  if (!field_ptr(field) || field == AMR_FIELD_W) return fail(AMR_E_ARG, "unknown field");
  const int64_t need = static_cast<int64_t>(in.tree.lastActive) * field_nv(field) * nn_;
  if (count < need) return fail(AMR_E_ARG, "buffer too small");
  return xfer(in, field, const_cast<double *>(src), true);
}

}  // namespace amr
