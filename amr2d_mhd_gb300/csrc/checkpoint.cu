// Checkpoint / restart of a handle and the reference's text writer
// (savedata.cpp:7-46).  Host code: the state comes through the same gather /
// scatter transfers as amr_download / amr_upload.
#include <cinttypes>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <iomanip>
#include <sstream>
#include <string>
#include <vector>

#include "engine.hpp"

namespace amr {

namespace {
constexpr char kMagic[8] = {'A', 'M', 'R', 'C', 'K', 'P', 'T', '1'};
// every pool of a block, in file order
constexpr int kFields[7] = {AMR_FIELD_U, AMR_FIELD_US, AMR_FIELD_FF, AMR_FIELD_GG,
                            AMR_FIELD_BI, AMR_FIELD_BIS, AMR_FIELD_EMF};

template <typename T>
bool put(std::ofstream &f, const T *p, size_t n) {
  f.write(reinterpret_cast<const char *>(p), static_cast<std::streamsize>(sizeof(T) * n));
  return static_cast<bool>(f);
}
template <typename T>
bool get(std::ifstream &f, T *p, size_t n) {
  f.read(reinterpret_cast<char *>(p), static_cast<std::streamsize>(sizeof(T) * n));
  return static_cast<bool>(f);
}
}  // namespace

// File: magic, ABI version, instance count, block edge; per instance the
// configuration, the time-loop counters, the quadtree and every field of
// blocks 0 .. lastActive-1 (float64, amr_download's layout).
int Engine::checkpoint_save(const char *path) {
  if (!initialised_) return fail(AMR_E_STATE, "amr_init has not been called");
  if (!path) return fail(AMR_E_ARG, "no path");
  std::ofstream f(path, std::ios::binary | std::ios::trunc);
  if (!f) return fail(AMR_E_ARG, std::string("cannot write ") + path);
  const int32_t head[4] = {AMR_ABI_VERSION, static_cast<int32_t>(inst_.size()), n_, 0};
  bool ok = put(f, kMagic, 8) && put(f, head, 4);
  std::vector<double> buf;
  for (Instance &in : inst_) {
    const Tree &t = in.tree;
    const double td[3] = {in.t, in.dt, in.dtn};
    const int64_t ti[3] = {in.count, in.cell_updates, in.done ? 1 : 0};
    const int32_t tr[4] = {t.lastActive, t.nbleafs, t.maxblocks(), 0};
    const uint64_t ver = t.version;
    ok = ok && put(f, &in.cfg, 1) && put(f, td, 3) && put(f, ti, 3) && put(f, tr, 4) && put(f, &ver, 1);
    ok = ok && put(f, t.lp.data(), static_cast<size_t>(t.lastActive)) &&
         put(f, t.icoord.data(), static_cast<size_t>(t.lastActive));
    const size_t mb = static_cast<size_t>(t.maxblocks());
    ok = ok && put(f, t.leafs.data(), mb) && put(f, t.iref.data(), mb) && put(f, t.icoarse.data(), mb);
    for (int fld : kFields) {
      buf.resize(static_cast<size_t>(t.lastActive) * field_nv(fld) * nn_);
      if (int rc = xfer(in, fld, buf.data(), false)) return rc;
      ok = ok && put(f, buf.data(), buf.size());
    }
  }
  if (!ok) return fail(AMR_E_ARG, std::string("write failed: ") + path);
  return AMR_OK;
}

// Restores a checkpoint into a handle created with the same configurations
// and not yet initialised; the next amr_step continues bit for bit.  A load
// that fails leaves every instance with a fresh tree, as amr_create made it.
int Engine::checkpoint_load(const char *path) {
  if (initialised_) return fail(AMR_E_STATE, "checkpoints load into a handle before amr_init");
  const int rc = checkpoint_read(path);
  if (rc != AMR_OK)
    for (Instance &in : inst_) in.tree = Tree(in.tree.shape());
  return rc;
}

int Engine::checkpoint_read(const char *path) {
  if (!path) return fail(AMR_E_ARG, "no path");
  std::ifstream f(path, std::ios::binary);
  if (!f) return fail(AMR_E_ARG, std::string("cannot read ") + path);
  char magic[8];
  int32_t head[4];
  if (!get(f, magic, 8) || std::memcmp(magic, kMagic, 8) != 0 || !get(f, head, 4))
    return fail(AMR_E_ARG, "not a checkpoint of this library");
  if (head[0] != AMR_ABI_VERSION || head[1] != static_cast<int32_t>(inst_.size()) || head[2] != n_)
    return fail(AMR_E_CONFIG, "checkpoint of a different handle shape");
  std::vector<double> buf;
  for (Instance &in : inst_) {
    amr_config c;
    double td[3];
    int64_t ti[3];
    int32_t tr[4];
    uint64_t ver;
    if (!get(f, &c, 1) || !get(f, td, 3) || !get(f, ti, 3) || !get(f, tr, 4) || !get(f, &ver, 1))
      return fail(AMR_E_ARG, "truncated checkpoint");
    if (std::memcmp(&c, &in.cfg, sizeof c) != 0) return fail(AMR_E_CONFIG, "checkpoint of a different configuration");
    Tree &t = in.tree;
    if (tr[2] != t.maxblocks() || tr[0] < 0 || tr[0] > t.maxblocks()) return fail(AMR_E_CONFIG, "bad tree size");
    t.lastActive = tr[0];
    t.nbleafs = tr[1];
    t.version = ver + 1;
    const size_t mb = static_cast<size_t>(t.maxblocks());
    if (!get(f, t.lp.data(), static_cast<size_t>(t.lastActive)) ||
        !get(f, t.icoord.data(), static_cast<size_t>(t.lastActive)) || !get(f, t.leafs.data(), mb) ||
        !get(f, t.iref.data(), mb) || !get(f, t.icoarse.data(), mb))
      return fail(AMR_E_ARG, "truncated checkpoint");
    std::string err;
    if (!t.check(err)) return fail(AMR_E_ARG, "corrupt checkpoint: " + err);
    in.t = td[0];
    in.dt = td[1];
    in.dtn = td[2];
    in.count = ti[0];
    in.cell_updates = ti[1];
    in.done = ti[2] != 0;
    if (int rc = assign_slots(in)) return rc;
    for (int fld : kFields) {
      buf.resize(static_cast<size_t>(t.lastActive) * field_nv(fld) * nn_);
      if (!get(f, buf.data(), buf.size())) return fail(AMR_E_ARG, "truncated checkpoint");
      if (int rc = xfer(in, fld, buf.data(), true)) return rc;
    }
  }
  programs_valid_ = false;
  initialised_ = true;
  return AMR_OK;
}

// savedata.cpp:7-46: one "#" header line per leaf block, then x, y, dx/2,
// dy/2 and the primitive state of every interior cell (j outer, i inner),
// columns of width 16; digits = 0 keeps the stream's default precision (6
// significant digits, as the reference), else setprecision(digits).
int Engine::save4py(int q, int id, const char *dir, int digits, char *name_out, size_t name_len) {
  if (!initialised_) return fail(AMR_E_STATE, "amr_init has not been called");
  if (q < 0 || q >= static_cast<int>(inst_.size()) || !dir) return fail(AMR_E_ARG, "bad instance or directory");
  Instance &in = inst_[q];
  const Tree &t = in.tree;
  std::vector<double> W(static_cast<size_t>(t.lastActive) * 8 * nn_);
  if (int rc = download(q, AMR_FIELD_W, W.data(), static_cast<int64_t>(W.size()))) return rc;
  std::ostringstream ss;
  ss << std::setw(3) << std::setfill('0') << id;
  const std::string name = std::string(dir) + "/" + in.cfg.ic + ss.str() + "t_" + std::to_string(in.t) + ".dat";
  std::ofstream out(name);
  if (!out) return fail(AMR_E_ARG, "cannot write " + name);
  if (digits > 0) out << std::setprecision(digits);
  // the reference's width of 16 holds 6 significant digits; wider columns
  // keep more digits separated
  const int w = digits > 9 ? digits + 9 : 16, ng = ng_, lo = ng, hi = ng + NI - 1;
  const double sx = in.cfg.geometry == 0 ? in.dx[0] : 0.0, sy = in.cfg.geometry == 0 ? in.dy[0] : 0.0;
  for (int nb = 0; nb < t.lastActive; nb++) {
    if (!t.leafs[nb]) continue;
    out << "#" << std::setw(w - 1) << "x" << std::setw(w) << "y" << std::setw(w) << "xdelta" << std::setw(w)
        << "ydelta" << std::setw(w) << "density" << std::setw(w) << "U" << std::setw(w) << "v" << std::setw(w)
        << "w" << std::setw(w) << "pressure" << std::setw(w) << "Bx" << std::setw(w) << "By" << std::setw(w)
        << "Bz" << "\n";
    const int lev = t.lp[nb][0];
    const double dx = in.dx[lev], dy = in.dy[lev];
    const double *wb = W.data() + static_cast<size_t>(nb) * 8 * nn_;
    for (int j = lo; j <= hi; j++) {
      const double y = ((j + t.icoord[nb][1] - ng) + 0.5) * dy - sy;
      for (int i = lo; i <= hi; i++) {
        const double x = ((i + t.icoord[nb][0] - ng) + 0.5) * dx - sx;
        out << std::setw(w) << x << std::setw(w) << y << std::setw(w) << dx / 2. << std::setw(w) << dy / 2.;
        for (int k = 0; k < 8; k++) out << std::setw(w) << wb[k * nn_ + j * n_ + i];
        out << "\n";
      }
    }
  }
  if (!out) return fail(AMR_E_ARG, "write failed: " + name);
  if (name_out && name_len) {
    std::strncpy(name_out, name.c_str(), name_len - 1);
    name_out[name_len - 1] = '\0';
  }
  return AMR_OK;
}

}  // namespace amr
