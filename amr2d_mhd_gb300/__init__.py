"""amr2d_mhd_gb300 — GB300 (sm_103a) per-block finite-volume update of a 2-D
block-structured AMR ideal-MHD solver, drop-in for the hot path of
spaceauk/AMR2D_MHD.

The compute path is the CUDA library libamr2d_mhd.so (C ABI in
include/amr2d_mhd.h); this module is a thin ctypes mirror of it.  There is no
CPU fallback: if the library is missing or no GPU is present the calls fail
with AmrError.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

from . import build as _build

__all__ = ["AmrError", "Config", "Simulation", "load", "FIELDS", "STATUS"]

HERE = os.path.dirname(os.path.abspath(__file__))
FIELDS = dict(U=0, Us=1, Bi=2, Bis=3, ff=4, gg=5, EMF=6, W=7)
STATUS = {0: "AMR_OK", -1: "AMR_E_CONFIG", -2: "AMR_E_CUDA", -3: "AMR_E_OOM", -4: "AMR_E_MAXBLOCKS",
          -5: "AMR_E_PRESSURE", -6: "AMR_E_NAN", -7: "AMR_E_DT", -8: "AMR_E_HLLC", -9: "AMR_E_STATE",
          -10: "AMR_E_TIMEOUT", -11: "AMR_E_UNSUPPORTED", -12: "AMR_E_ARG", -13: "AMR_E_TOO_LARGE"}

# every entry point declared in include/amr2d_mhd.h
EXPORTS = ["amr_config_default", "amr_config_from_input", "amr_config_blast", "amr_config_kh", "amr_abi_version", "amr_status_string",
           "amr_create", "amr_create_batch", "amr_destroy", "amr_set_stream", "amr_last_error",
           "amr_init", "amr_step", "amr_step_begin", "amr_step_end", "amr_run", "amr_get_info", "amr_locate_bounds", "amr_boundary",
           "amr_muscl2d_rk", "amr_ct2d", "amr_cfl_dt", "amr_admesh", "amr_get_tree", "amr_set_tree", "amr_download",
           "amr_upload", "amr_profile_enable", "amr_profile_read", "amr_cfl_dt_static", "amr_riemann", "amr_criteria", "amr_criteria_flags", "amr_admesh_marked", "amr_set_remesh", "amr_autotune", "amr_save4py",
           "amr_checkpoint_save", "amr_checkpoint_load", "amr_adjoint_enable",
           "amr_adjoint_seed", "amr_adjoint_step", "amr_adjoint_read", "amr_adjoint_recorded"]


class AmrError(RuntimeError):
    def __init__(self, code, msg=""):
        super().__init__("%s (%d): %s" % (STATUS.get(code, "?"), code, msg))
        self.code = code


class Config(ctypes.Structure):
    _fields_ = [("struct_size", ctypes.c_int32), ("nx", ctypes.c_int32), ("ny", ctypes.c_int32),
                ("nvar", ctypes.c_int32), ("lenx", ctypes.c_double), ("leny", ctypes.c_double),
                ("cfl", ctypes.c_double), ("ic", ctypes.c_char * 16), ("limiter", ctypes.c_char * 16),
                ("flux", ctypes.c_char * 16), ("maxlevs", ctypes.c_int32), ("nghosts", ctypes.c_int32),
                ("nroots_x", ctypes.c_int32), ("nroots_y", ctypes.c_int32), ("periodic", ctypes.c_int32),
                ("geometry", ctypes.c_int32), ("gamma", ctypes.c_double), ("t_end", ctypes.c_double),
                ("ic_param", ctypes.c_double * 24), ("precision", ctypes.c_int32),
                ("reserved0", ctypes.c_int32), ("dt_fixed", ctypes.c_double), ("ct_type", ctypes.c_int32),
                ("diffusion", ctypes.c_int32), ("reserved", ctypes.c_int32 * 2)]


class Info(ctypes.Structure):
    _fields_ = [("t", ctypes.c_double), ("dt", ctypes.c_double), ("dt_next", ctypes.c_double),
                ("t_end", ctypes.c_double), ("gamma", ctypes.c_double), ("steps", ctypes.c_int64),
                ("last_active", ctypes.c_int32), ("n_leaves", ctypes.c_int32), ("nb_leafs", ctypes.c_int32),
                ("done", ctypes.c_int32), ("n_instances", ctypes.c_int32), ("nx_tot", ctypes.c_int32),
                ("ny_tot", ctypes.c_int32), ("cell_updates", ctypes.c_int64)]


class Profile(ctypes.Structure):
    _fields_ = [("launches", ctypes.c_int64), ("stage_launches", ctypes.c_int64), ("stage_ms", ctypes.c_double),
                ("stage_cells", ctypes.c_int64), ("h2d_bytes", ctypes.c_int64), ("d2h_bytes", ctypes.c_int64),
                ("host_compile_ms", ctypes.c_double), ("host_admesh_ms", ctypes.c_double),
                ("wait_ms", ctypes.c_double), ("steps", ctypes.c_int64), ("step_gpu_ms", ctypes.c_double),
                ("host_capture_ms", ctypes.c_double)]


_lib = None


def load(build_if_missing: bool = True):
    """Load libamr2d_mhd.so (building it when the sources are newer)."""
    global _lib
    if _lib is not None:
        return _lib
    path = _build.LIB
    if build_if_missing:
        path = _build.build()
    if not os.path.exists(path):
        raise ImportError("libamr2d_mhd.so is not built (%s); run __graft_entry__.build()" % path)
    L = ctypes.CDLL(path)
    vp, i32, i64, dp = ctypes.c_void_p, ctypes.c_int32, ctypes.c_int64, ctypes.c_void_p
    sig = {
        "amr_config_default": (None, [ctypes.POINTER(Config)]),
        "amr_config_from_input": (ctypes.c_int, [ctypes.c_char_p, ctypes.POINTER(Config)]),
        "amr_config_blast": (ctypes.c_int, [ctypes.c_uint64, i32, ctypes.POINTER(Config)]),
        "amr_config_kh": (ctypes.c_int, [ctypes.c_uint64, ctypes.POINTER(Config)]),
        "amr_abi_version": (ctypes.c_int, []),
        "amr_status_string": (ctypes.c_char_p, [ctypes.c_int]),
        "amr_create": (ctypes.c_int, [ctypes.POINTER(Config), ctypes.POINTER(vp)]),
        "amr_create_batch": (ctypes.c_int, [ctypes.POINTER(Config), i32, ctypes.POINTER(vp)]),
        "amr_destroy": (ctypes.c_int, [vp]),
        "amr_set_stream": (ctypes.c_int, [vp, vp]),
        "amr_last_error": (ctypes.c_int, [vp, ctypes.c_char_p, ctypes.c_size_t]),
        "amr_init": (ctypes.c_int, [vp]),
        "amr_step": (ctypes.c_int, [vp]),
        "amr_step_begin": (ctypes.c_int, [vp]),
        "amr_step_end": (ctypes.c_int, [vp]),
        "amr_run": (ctypes.c_int, [vp, i64]),
        "amr_get_info": (ctypes.c_int, [vp, i32, ctypes.POINTER(Info)]),
        "amr_locate_bounds": (ctypes.c_int, [vp]),
        "amr_boundary": (ctypes.c_int, [vp, i32]),
        "amr_muscl2d_rk": (ctypes.c_int, [vp, i32]),
        "amr_ct2d": (ctypes.c_int, [vp, i32]),
        "amr_cfl_dt": (ctypes.c_int, [vp, ctypes.POINTER(ctypes.c_double)]),
        "amr_admesh": (ctypes.c_int, [vp]),
        "amr_get_tree": (ctypes.c_int, [vp, i32, dp, dp, dp, i32]),
        "amr_set_tree": (ctypes.c_int, [vp, i32, i32, i32, dp, dp, dp, ctypes.c_double, ctypes.c_double,
                                        ctypes.c_double, i64]),
        "amr_download": (ctypes.c_int, [vp, i32, i32, dp, i64]),
        "amr_upload": (ctypes.c_int, [vp, i32, i32, dp, i64]),
        "amr_profile_enable": (ctypes.c_int, [vp, i32]),
        "amr_set_remesh": (ctypes.c_int, [vp, i32]),
        "amr_profile_read": (ctypes.c_int, [vp, ctypes.POINTER(Profile)]),
        "amr_cfl_dt_static": (ctypes.c_int, [dp, i32, i32, dp, ctypes.c_double, dp, vp]),
        "amr_riemann": (ctypes.c_int, [i32, i32, i32, ctypes.c_double, dp, dp, dp, vp, ctypes.c_int64]),
        "amr_criteria": (ctypes.c_int, [vp, dp, i32]),
        "amr_criteria_flags": (ctypes.c_int, [vp, dp, dp, i32]),
        "amr_admesh_marked": (ctypes.c_int, [vp, dp, dp, i32]),
        "amr_autotune": (ctypes.c_int, [vp, i32, ctypes.c_char_p, ctypes.c_size_t]),
        "amr_save4py": (ctypes.c_int, [vp, i32, i32, ctypes.c_char_p, i32, ctypes.c_char_p, ctypes.c_size_t]),
        "amr_checkpoint_save": (ctypes.c_int, [vp, ctypes.c_char_p]),
        "amr_checkpoint_load": (ctypes.c_int, [vp, ctypes.c_char_p]),
        "amr_adjoint_enable": (ctypes.c_int, [vp, i32]),
        "amr_adjoint_seed": (ctypes.c_int, [vp, i32, i32, dp, i64]),
        "amr_adjoint_step": (ctypes.c_int, [vp]),
        "amr_adjoint_read": (ctypes.c_int, [vp, i32, i32, dp, i64]),
        "amr_adjoint_recorded": (ctypes.c_int, [vp, ctypes.POINTER(i32)]),
    }
    for name, (res, args) in sig.items():
        fn = getattr(L, name)
        fn.restype = res
        fn.argtypes = args
    _lib = L
    return L


def make_config(ic="rotor", limiter="MC", flux="RUSA", cfl=0.5, maxlevs=5, nghosts=2, nroots=(2, 2),
                periodic=False, geometry=0, gamma=0.0, t_end=0.0, ic_param=None, precision="fp64",
                lenx=1.0, leny=1.0, nx=16, ny=16, input_txt=None, ct_type=1, diffusion=False) -> Config:
    """An amr_config; defaults are the reference's input.txt and defs.hpp."""
    L = load()
    c = Config()
    L.amr_config_default(ctypes.byref(c))
    if input_txt is not None:
        rc = L.amr_config_from_input(os.fsencode(input_txt), ctypes.byref(c))
        if rc:
            raise AmrError(rc, "cannot read %s" % input_txt)
    else:
        c.nx, c.ny, c.lenx, c.leny, c.cfl = nx, ny, lenx, leny, cfl
        # zero-padded, as the C side writes names (configurations are
        # compared byte for byte, e.g. by amr_checkpoint_load); a ctypes
        # char-array field assignment stops at the first NUL
        for field, name in (("ic", ic), ("limiter", limiter), ("flux", flux)):
            ctypes.memset(ctypes.addressof(c) + getattr(Config, field).offset, 0, 16)
            setattr(c, field, name.encode()[:15])
    c.maxlevs, c.nghosts = maxlevs, nghosts
    c.nroots_x, c.nroots_y = nroots
    c.periodic, c.geometry = int(periodic), int(geometry)
    c.gamma, c.t_end = gamma, t_end
    for i, v in enumerate(ic_param or []):
        c.ic_param[i] = v
    c.precision = {"fp64": 0, "fp32": 1}[precision]
    c.ct_type, c.diffusion = ct_type, int(diffusion)
    return c


def blast_config(seed, index, precision="fp64") -> Config:
    """Instance `index` of the seeded cylindrical blast batch (amr_config_blast)."""
    c = Config()
    rc = load().amr_config_blast(seed, index, ctypes.byref(c))
    if rc:
        raise AmrError(rc, "amr_config_blast")
    c.precision = {"fp64": 0, "fp32": 1}[precision]
    return c


def riemann(flux, wL, wR, gamma, dir_y=False, mag_field=True):
    """riemannS (riemannS.cpp:7-56) on the GPU (amr_riemann) for arrays of
    face states wL, wR [n, 8]; returns (fluxes [n, 8], status [n])."""
    wL = np.ascontiguousarray(np.atleast_2d(wL), np.float64)
    wR = np.ascontiguousarray(np.atleast_2d(wR), np.float64)
    if wL.shape != wR.shape or wL.shape[1] != 8:
        raise ValueError("wL, wR: [n, 8] arrays of the same shape")
    out = np.zeros_like(wL)
    st = np.zeros(len(wL), np.int32)
    names = ["RUSA", "HLLE", "HLLC", "HLLD", "ROE"]
    fl = names.index(flux) if isinstance(flux, str) else int(flux)
    rc = load().amr_riemann(fl, int(bool(dir_y)), int(bool(mag_field)), float(gamma), wL.ctypes.data,
                            wR.ctypes.data, out.ctypes.data, st.ctypes.data, len(wL))
    if rc:
        raise AmrError(rc, "amr_riemann")
    return out, st


def kh_config(seed, precision="fp64") -> Config:
    """The frozen-mesh Kelvin-Helmholtz problem of amr_config_kh."""
    c = Config()
    rc = load().amr_config_kh(seed, ctypes.byref(c))
    if rc:
        raise AmrError(rc, "amr_config_kh")
    c.precision = {"fp64": 0, "fp32": 1}[precision]
    return c


def ot_config(maxlevs=7, precision="fp64", cfl=0.4, limiter="WENO5", dt_fixed=0.0) -> Config:
    """Orszag-Tang vortex on [0, 2 pi]^2, periodic, 4 x 4 roots of 16 x 16,
    WENO5 (4 ghost layers) or a MUSCL limiter (2) + HLLD, gamma 5/3, t_end pi
    (extension); dt_fixed > 0 replaces the CFL step (a common time grid for
    comparing precisions)."""
    import math
    c = make_config(ic="OT", limiter=limiter, flux="HLLD", cfl=cfl, maxlevs=maxlevs,
                    nghosts=4 if limiter == "WENO5" else 2, nroots=(4, 4), periodic=True, geometry=1,
                    gamma=5.0 / 3.0, t_end=math.pi, precision=precision, lenx=2 * math.pi, leny=2 * math.pi)
    c.dt_fixed = dt_fixed
    return c


class Simulation:
    """One handle: an AMR problem (or a batch of them) resident on the GPU.

    The methods mirror the reference's seam: init() is basegrid + IC2Dtype +
    the initial admesh, step() one iteration of main.cpp's time loop, and
    boundary / MUSCL2D / CT2D / cfl_dt / admesh the individual calls.
    """

    def __init__(self, configs=None, **kw):
        L = load()
        if configs is None:
            configs = [make_config(**kw)]
        elif isinstance(configs, Config):
            configs = [configs]
        arr = (Config * len(configs))(*configs)
        h = ctypes.c_void_p()
        rc = L.amr_create_batch(arr, len(configs), ctypes.byref(h))
        if rc:
            raise AmrError(rc, "amr_create failed")
        self.h = h
        self.n = len(configs)
        self.configs = [Config.from_buffer_copy(c) for c in configs]

    def close(self):
        if getattr(self, "h", None):
            load().amr_destroy(self.h)
            self.h = None

    __del__ = close

    def _ck(self, rc):
        if rc:
            buf = ctypes.create_string_buffer(512)
            load().amr_last_error(self.h, buf, 512)
            raise AmrError(rc, buf.value.decode(errors="replace"))

    def init(self):
        self._ck(load().amr_init(self.h))
        return self

    def step(self):
        self._ck(load().amr_step(self.h))

    def step_begin(self):
        """Launch one step's device work and return (amr_step_begin)."""
        self._ck(load().amr_step_begin(self.h))

    def step_end(self):
        """Finish the step in flight: wait, advance t / dt, remesh (amr_step_end)."""
        self._ck(load().amr_step_end(self.h))

    def run(self, max_steps=-1):
        self._ck(load().amr_run(self.h, max_steps))

    def info(self, instance=0):
        inf = Info()
        self._ck(load().amr_get_info(self.h, instance, ctypes.byref(inf)))
        return {k: getattr(inf, k) for k, _ in Info._fields_}

    # reference-function entry points
    def locate_bounds(self):
        self._ck(load().amr_locate_bounds(self.h))

    def boundary(self, field):
        self._ck(load().amr_boundary(self.h, FIELDS[field]))

    def MUSCL2D(self, step):
        self._ck(load().amr_muscl2d_rk(self.h, step))

    def CT2D(self, step):
        self._ck(load().amr_ct2d(self.h, step))

    def cfl_dt(self):
        v = ctypes.c_double()
        self._ck(load().amr_cfl_dt(self.h, ctypes.byref(v)))
        return v.value

    def admesh(self):
        self._ck(load().amr_admesh(self.h))

    def set_remesh(self, on):
        """on=False: step() stops before main.cpp's closing admesh; call
        admesh() after acting on the state (amr_set_remesh)."""
        self._ck(load().amr_set_remesh(self.h, int(bool(on))))

    # state exchange
    def tree(self, instance=0):
        na = self.info(instance)["last_active"]
        lp = np.zeros((na, 8), np.int32)
        ic = np.zeros((na, 2), np.int32)
        lf = np.zeros(na, np.uint8)
        self._ck(load().amr_get_tree(self.h, instance, lp.ctypes.data, ic.ctypes.data, lf.ctypes.data, na))
        return lp, ic, lf.astype(bool)

    def set_tree(self, lp, icoord, leafs, nb_leafs, t, dt, dt_next, steps, instance=0):
        """Take over the quadtree and time state of a run (amr_set_tree), in
        place of init(); then upload U, Bi (and ff, gg) before stepping."""
        lp = np.ascontiguousarray(lp, np.int32)
        ic = np.ascontiguousarray(icoord, np.int32)
        lf = np.ascontiguousarray(np.asarray(leafs).astype(np.uint8))
        self._ck(load().amr_set_tree(self.h, instance, lp.shape[0], int(nb_leafs), lp.ctypes.data, ic.ctypes.data,
                                     lf.ctypes.data, float(t), float(dt), float(dt_next), int(steps)))
        return self

    def download(self, field, instance=0, out=None):
        """Blocks 0..last_active-1 of `field` as float64 [block][var][j][i];
        into `out` when it is a C-contiguous float64 array of that shape."""
        inf = self.info(instance)
        nv = {"Bi": 2, "Bis": 2, "EMF": 1}.get(field, 8)
        n = inf["nx_tot"]
        shape = (inf["last_active"], nv, n, n)
        if (out is not None and out.shape == shape and out.dtype == np.float64
                and out.flags["C_CONTIGUOUS"] and out.flags["WRITEABLE"]):
            a = out
        else:
            a = np.empty(shape, np.float64)
        self._ck(load().amr_download(self.h, instance, FIELDS[field], a.ctypes.data, a.size))
        return a

    def upload(self, field, arr, instance=0):
        a = np.ascontiguousarray(arr, np.float64)
        self._ck(load().amr_upload(self.h, instance, FIELDS[field], a.ctypes.data, a.size))

    def set_stream(self, stream_ptr):
        """Issue this handle's work on an existing CUDA stream (e.g. torch's)."""
        self._ck(load().amr_set_stream(self.h, ctypes.c_void_p(stream_ptr)))

    def profile(self, enable=None):
        """profile(True/False) resets the counters (and turns the stage-kernel
        events on/off); profile() returns the counters."""
        if enable is not None:
            self._ck(load().amr_profile_enable(self.h, int(enable)))
            return None
        p = Profile()
        self._ck(load().amr_profile_read(self.h, ctypes.byref(p)))
        return {k: getattr(p, k) for k, _ in Profile._fields_}

    def uniform(self, var=0, level=None, instance=0, field="U"):
        """Variable `var` of the leaf blocks painted piecewise constant onto
        the uniform grid of `level` (default: the finest level); [i][j]."""
        c = self.configs[instance]
        ng = c.nghosts
        lp, ic, lf = self.tree(instance)
        if level is None:
            level = c.maxlevs - 1
        a = self.download(field, instance)
        nx, ny = c.nx * c.nroots_x * 2 ** level, c.ny * c.nroots_y * 2 ** level
        out = np.zeros((nx, ny))
        for b in np.nonzero(lf)[0]:
            r = 2 ** (level - lp[b, 0])
            if r < 1:
                raise ValueError("level is coarser than a leaf")
            v = a[b, var, ng:-ng, ng:-ng].T
            x0, y0 = ic[b, 0] * r, ic[b, 1] * r
            out[x0:x0 + c.nx * r, y0:y0 + c.ny * r] = np.kron(v, np.ones((r, r)))
        return out

    def criteria(self):
        """criteria.cpp per block ID of instance 0 (-1 for non-leaves)."""
        na = self.info()["last_active"]
        g = np.empty(na, np.float64)
        self._ck(load().amr_criteria(self.h, g.ctypes.data, na))
        return g

    def criteria_flags(self):
        """(iref, icoarse) of criteria.cpp per block ID (amr_criteria_flags)."""
        na = self.info()["last_active"]
        iref = np.zeros(na, np.uint8)
        ico = np.zeros(na, np.uint8)
        self._ck(load().amr_criteria_flags(self.h, iref.ctypes.data, ico.ctypes.data, na))
        return iref.astype(bool), ico.astype(bool)

    def admesh_marked(self, iref, icoarse):
        """admesh with the caller's refine / coarsen marks per block ID
        (amr_admesh_marked)."""
        na = self.info()["last_active"]
        r = np.ascontiguousarray(np.asarray(iref, dtype=bool)[:na], np.uint8)
        c = np.ascontiguousarray(np.asarray(icoarse, dtype=bool)[:na], np.uint8)
        if r.size < na or c.size < na:
            raise ValueError("need a mark per block ID (%d)" % na)
        self._ck(load().amr_admesh_marked(self.h, r.ctypes.data, c.ctypes.data, na))

    def autotune(self, reps=5):
        """Pick the fastest launch schedule on the current state; returns the
        report (one line per candidate, the chosen one marked '*')."""
        buf = ctypes.create_string_buffer(8192)
        self._ck(load().amr_autotune(self.h, reps, buf, 8192))
        return buf.value.decode()

    def save4py(self, directory, id=0, digits=0, instance=0):
        """savedata.cpp's text output of one instance; returns the file name."""
        buf = ctypes.create_string_buffer(4096)
        self._ck(load().amr_save4py(self.h, instance, id, os.fsencode(directory), digits, buf, 4096))
        return buf.value.decode()

    def checkpoint_save(self, path):
        self._ck(load().amr_checkpoint_save(self.h, os.fsencode(path)))

    def checkpoint_load(self, path):
        """Restore a checkpoint instead of init() (same configurations)."""
        self._ck(load().amr_checkpoint_load(self.h, os.fsencode(path)))
        return self

    # discrete adjoint of the frozen-mesh step
    def adjoint_enable(self, on=True):
        self._ck(load().amr_adjoint_enable(self.h, int(on)))

    def adjoint_seed(self, field, lam, instance=0):
        a = np.ascontiguousarray(lam, np.float64)
        self._ck(load().amr_adjoint_seed(self.h, instance, FIELDS[field], a.ctypes.data, a.size))

    def adjoint_step(self):
        self._ck(load().amr_adjoint_step(self.h))

    def adjoint_read(self, field, instance=0):
        inf = self.info(instance)
        nv = 2 if field == "Bi" else 8
        n = inf["nx_tot"]
        a = np.empty((inf["last_active"], nv, n, n), np.float64)
        self._ck(load().amr_adjoint_read(self.h, instance, FIELDS[field], a.ctypes.data, a.size))
        return a

    def adjoint_recorded(self):
        n = ctypes.c_int32()
        self._ck(load().amr_adjoint_recorded(self.h, ctypes.byref(n)))
        return n.value

    def state(self, instance=0):
        """Dict in the form the oracle's state() returns."""
        inf = self.info(instance)
        lp, ic, lf = self.tree(instance)
        return dict(t=inf["t"], dt=inf["dt"], step=inf["steps"], lastActive=inf["last_active"],
                    nbleafs=inf["nb_leafs"], lp=lp, icoord=ic, leafs=lf, U=self.download("U", instance),
                    Bi=self.download("Bi", instance))
