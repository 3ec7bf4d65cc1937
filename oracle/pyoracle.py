"""Test infrastructure, not product code.

ctypes binding of the oracle (oracle/amr_oracle.c), the CPU FP64 restatement
of spaceauk/AMR2D_MHD's time loop, plus a reader for the full-precision state
dumps written by the reference build (oracle/ref.mk + oracle/ref_hook.cpp).

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg import
this module.
"""
from __future__ import annotations

import ctypes
import os
import struct
import subprocess
from dataclasses import dataclass

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "liboracle.so")

LIMITERS = ["1st", "noSL", "minmod", "VanLeer", "Superbee", "MC", "Koren", "Cada3rd",
            "WENO3", "WENO5"]
FLUXES = ["RUSA", "HLLE", "HLLC", "HLLD", "ROE"]
ICS = ["SST", "SST1", "SSTy", "BWx", "BWx1", "BWy", "BWy1", "rotor", "rotor_b", "OT",
       "blast", "KH"]
GET = dict(U=0, Us=1, W=2, ff=3, gg=4, Bi=5, Bis=6, EMF=7, lp=8, icoord=9, leafs=10)


def build(force: bool = False) -> str:
    """Compile the oracle with the host C compiler (no FMA contraction)."""
    src = os.path.join(HERE, "amr_oracle.c")
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= max(
            os.path.getmtime(src), os.path.getmtime(os.path.join(HERE, "amr_oracle.h"))):
        return LIB
    os.makedirs(BUILD, exist_ok=True)
    tmp = LIB + ".tmp%d" % os.getpid()
    cmd = ["gcc", "-O2", "-std=c11", "-ffp-contract=off", "-fopenmp", "-fPIC", "-shared",
           src, "-o", tmp, "-lm"]
    subprocess.check_call(cmd)
    os.replace(tmp, LIB)
    return LIB


class _Cfg(ctypes.Structure):
    _fields_ = [("nx_int", ctypes.c_int), ("ny_int", ctypes.c_int), ("nghosts", ctypes.c_int),
                ("maxlevs", ctypes.c_int), ("nroots_x", ctypes.c_int), ("nroots_y", ctypes.c_int),
                ("periodic", ctypes.c_int), ("geom_ref", ctypes.c_int),
                ("lenx", ctypes.c_double), ("leny", ctypes.c_double), ("cfl", ctypes.c_double),
                ("ic", ctypes.c_int), ("limiter", ctypes.c_int), ("flux", ctypes.c_int),
                ("gamma_override", ctypes.c_double), ("tend_override", ctypes.c_double),
                ("ic_param", ctypes.c_double * 24), ("nthreads", ctypes.c_int), ("dt_fixed", ctypes.c_double),
                ("ct_type", ctypes.c_int), ("diffusion", ctypes.c_int)]


_lib = None


def lib():
    global _lib
    if _lib is None:
        _lib = ctypes.CDLL(build())
        L = _lib
        L.oracle_create.restype = ctypes.c_void_p
        L.oracle_create.argtypes = [ctypes.POINTER(_Cfg)]
        L.oracle_destroy.argtypes = [ctypes.c_void_p]
        L.oracle_init.argtypes = [ctypes.c_void_p]
        L.oracle_step.argtypes = [ctypes.c_void_p]
        L.oracle_run.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_double]
        L.oracle_done.argtypes = [ctypes.c_void_p]
        L.oracle_info.argtypes = [ctypes.c_void_p, ctypes.POINTER(ctypes.c_int),
                                  ctypes.POINTER(ctypes.c_double)]
        L.oracle_get.restype = ctypes.c_int64
        L.oracle_get.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p]
        L.oracle_set.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p]
        L.oracle_error.restype = ctypes.c_char_p
        L.oracle_error.argtypes = [ctypes.c_void_p]
        L.oracle_set_remesh.argtypes = [ctypes.c_void_p, ctypes.c_int]
        L.oracle_admesh.argtypes = [ctypes.c_void_p]
        L.oracle_admesh_marked.argtypes = [ctypes.c_void_p] * 3
        L.oracle_fill.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int, ctypes.c_int]
        L.oracle_slopelimiter.restype = ctypes.c_double
        L.oracle_slopelimiter.argtypes = [ctypes.c_int, ctypes.c_double, ctypes.c_double]
        L.oracle_riemann.argtypes = [ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p,
                                     ctypes.c_double, ctypes.c_int, ctypes.c_void_p]
        L.oracle_riemann_mf.argtypes = [ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p,
                                        ctypes.c_double, ctypes.c_int, ctypes.c_int, ctypes.c_void_p]
        L.oracle_wavespeeds.argtypes = [ctypes.c_void_p, ctypes.c_double, ctypes.c_int,
                                        ctypes.c_void_p]
    return _lib


class OracleError(RuntimeError):
    pass


class Oracle:
    """One AMR problem advanced by the oracle."""

    def __init__(self, ic="BWx", limiter="MC", flux="RUSA", cfl=0.4, maxlevs=4, nx=16, ny=16,
                 nghosts=2, nroots=(2, 2), periodic=False, geom_ref=True, lenx=1.0, leny=1.0,
                 gamma=0.0, tend=0.0, ic_param=None, nthreads=1, dt_fixed=0.0, ct_type=1, diffusion=False):
        c = _Cfg()
        c.nx_int, c.ny_int, c.nghosts, c.maxlevs = nx, ny, nghosts, maxlevs
        c.nroots_x, c.nroots_y = nroots
        c.periodic, c.geom_ref = int(periodic), int(geom_ref)
        c.lenx, c.leny, c.cfl = lenx, leny, cfl
        c.ic, c.limiter, c.flux = ICS.index(ic), LIMITERS.index(limiter), FLUXES.index(flux)
        c.gamma_override, c.tend_override = gamma, tend
        for i, v in enumerate(ic_param or []):
            c.ic_param[i] = v
        c.nthreads = nthreads
        c.dt_fixed = dt_fixed
        c.ct_type, c.diffusion = ct_type, int(diffusion)
        self._cfg = c
        self.h = lib().oracle_create(ctypes.byref(c))
        if not self.h:
            raise OracleError("oracle_create failed")
        self.nx, self.ny = nx + 2 * nghosts, ny + 2 * nghosts

    def __del__(self):
        if getattr(self, "h", None):
            lib().oracle_destroy(self.h)
            self.h = None

    def _check(self, rc):
        if rc != 0:
            raise OracleError(lib().oracle_error(self.h).decode())

    def init(self):
        self._check(lib().oracle_init(self.h))
        return self

    def step(self):
        self._check(lib().oracle_step(self.h))

    def run(self, nsteps=-1, t_stop=-1.0):
        self._check(lib().oracle_run(self.h, nsteps, t_stop))

    @property
    def done(self):
        return bool(lib().oracle_done(self.h))

    def info(self):
        ints = (ctypes.c_int * 8)()
        dbls = (ctypes.c_double * 8)()
        lib().oracle_info(self.h, ints, dbls)
        return dict(lastActive=ints[0], nbleafs=ints[1], count=ints[2], maxblocks=ints[5],
                    t=dbls[0], dt=dbls[1], dt_next=dbls[2], gamma=dbls[3], tEnd=dbls[4],
                    dx0=dbls[5], dy0=dbls[6])

    def get(self, what):
        L = lib()
        n = L.oracle_get(self.h, GET[what], None)
        na = self.info()["lastActive"]
        if what in ("lp", "icoord"):
            a = np.empty(n, np.int32)
            L.oracle_get(self.h, GET[what], a.ctypes.data)
            return a.reshape(na, -1)
        if what == "leafs":
            a = np.empty(n, np.uint8)
            L.oracle_get(self.h, GET[what], a.ctypes.data)
            return a.astype(bool)
        a = np.empty(n, np.float64)
        L.oracle_get(self.h, GET[what], a.ctypes.data)
        nv = {"Bi": 2, "Bis": 2, "EMF": 1}.get(what, 8)
        return a.reshape(na, nv, self.ny, self.nx)

    def set(self, what, arr):
        a = np.ascontiguousarray(arr, dtype=np.float64)
        self._check(lib().oracle_set(self.h, GET[what], a.ctypes.data))

    def set_remesh(self, on):
        lib().oracle_set_remesh(self.h, int(on))

    def admesh(self):
        self._check(lib().oracle_admesh(self.h))

    def admesh_marked(self, iref, icoarse):
        """admesh with the caller's marks per block ID (criteria's place)."""
        n = self.info()["lastActive"]
        r = np.ascontiguousarray(np.asarray(iref, bool)[:n], np.uint8)
        c = np.ascontiguousarray(np.asarray(icoarse, bool)[:n], np.uint8)
        assert r.size == n and c.size == n
        self._check(lib().oracle_admesh_marked(self.h, r.ctypes.data, c.ctypes.data))

    def fill(self, field, kind):
        """Sequential ghost fill (kind 0 cell, 1 face, 2 edge) of a copy of `field`."""
        a = np.array(field, dtype=np.float64, order="C", copy=True)
        lib().oracle_fill(self.h, a.ctypes.data, a.shape[1], kind)
        return a

    def state(self):
        """Dict in the same form as read_ref_dump()."""
        inf = self.info()
        return dict(t=inf["t"], dt=inf["dt"], step=inf["count"], lastActive=inf["lastActive"],
                    nbleafs=inf["nbleafs"], lp=self.get("lp"), icoord=self.get("icoord"),
                    leafs=self.get("leafs"), U=self.get("U"), W=self.get("W"), Bi=self.get("Bi"))


def slopelimiter(limiter, r, eta=0.0):
    return lib().oracle_slopelimiter(LIMITERS.index(limiter), r, eta)


def riemann(flux, wL, wR, gamma, dir_y=False, mag_field=True):
    """riemannS.cpp:7-56; mag_field = the reference's compile-time MAG_field
    (defs.hpp:32), False for its hydrodynamic configuration (where ROE runs)."""
    a = np.ascontiguousarray(wL, np.float64)
    b = np.ascontiguousarray(wR, np.float64)
    out = np.zeros(8)
    rc = lib().oracle_riemann_mf(FLUXES.index(flux), a.ctypes.data, b.ctypes.data, gamma,
                                 int(dir_y), int(bool(mag_field)), out.ctypes.data)
    if rc != 0:
        raise OracleError("riemann rc=%d" % rc)
    return out


def read_ref_dump(path):
    """Read a state dump of the reference build (format: oracle/ref_hook.cpp)."""
    with open(path, "rb") as f:
        buf = f.read()
    if buf[:8] != b"AMRREF01":
        raise ValueError("not a reference dump: %s" % path)
    nx, ny, nvar, maxlevs, ng, na, nbleafs, step = struct.unpack_from("<8i", buf, 8)
    t, dt, gamma, dx0, dy0 = struct.unpack_from("<5d", buf, 40)
    off = 80
    meta = np.frombuffer(buf, np.int32, na * 11, off).reshape(na, 11)
    off += na * 11 * 4
    ncell = na * nvar * ny * nx
    U = np.frombuffer(buf, np.float64, ncell, off).reshape(na, nvar, ny, nx)
    off += ncell * 8
    W = np.frombuffer(buf, np.float64, ncell, off).reshape(na, nvar, ny, nx)
    off += ncell * 8
    Bi = np.frombuffer(buf, np.float64, na * 2 * ny * nx, off).reshape(na, 2, ny, nx)
    return dict(t=t, dt=dt, step=step, lastActive=na, nbleafs=nbleafs, maxlevs=maxlevs,
                gamma=gamma, dx0=dx0, lp=meta[:, :8].copy(), icoord=meta[:, 8:10].copy(),
                leafs=meta[:, 10].astype(bool), U=U.copy(), W=W.copy(), Bi=Bi.copy())


def criteria_grad(W, ng=2):
    """criteria.cpp:11-29 per block: max over interior cells of the relative
    jumps of p, rho, Bx, By (W: [blocks][8][n][n])."""
    n = W.shape[-1]
    out = np.zeros(W.shape[0])
    c = slice(ng, n - ng)
    for k in (4, 0, 5, 6):
        w = W[:, k]
        w0 = w[:, c, c]
        d = np.abs(w[:, c, ng + 1:n - ng + 1] - w0)
        d = np.maximum(d, np.abs(w[:, c, ng - 1:n - ng - 1] - w0))
        d = np.maximum(d, np.abs(w[:, ng + 1:n - ng + 1, c] - w0))
        d = np.maximum(d, np.abs(w[:, ng - 1:n - ng - 1, c] - w0))
        r = d / np.maximum(1e-15, np.abs(w0))
        out = np.maximum(out, r.reshape(W.shape[0], -1).max(axis=1))
    return out


def criteria_flags(grad, leafs, level, maxlevs, r_thresh=0.05, c_thresh=1.0):
    """criteria.cpp:31-43: refine a leaf whose criterion reaches r_thresh below
    the finest level; coarsen a leaf whose criterion stays below r_thresh and
    at most c_thresh (before the neighbour rule of critneighup.cpp)."""
    iref = leafs & (grad >= r_thresh) & (level < maxlevs - 1)
    icoarse = leafs & (grad < r_thresh) & (grad <= c_thresh)
    return iref, icoarse


def compare_states(a, b, ng=2):
    """Compare two states (dicts as above) on the leaf blocks.

    Returns (same_tree, max_abs_diff_U, max_rel_L1_per_var, max_abs_diff_Bi).  The
    comparison is by block ID, which both implementations assign identically.
    """
    same_tree = (a["lastActive"] == b["lastActive"] and np.array_equal(a["leafs"], b["leafs"])
                 and np.array_equal(a["lp"], b["lp"]) and np.array_equal(a["icoord"], b["icoord"]))
    if not same_tree:
        return False, np.inf, np.full(8, np.inf), np.inf
    lf = a["leafs"]
    sl = (slice(None), slice(None), slice(ng, -ng), slice(ng, -ng))
    ua, ub = a["U"][lf][sl], b["U"][lf][sl]
    dU = np.abs(ua - ub)
    rel = dU.sum(axis=(0, 2, 3)) / np.maximum(np.abs(ub).sum(axis=(0, 2, 3)), 1e-300)
    dB = np.abs(a["Bi"][lf] - b["Bi"][lf]).max() if lf.any() else 0.0
    return True, float(dU.max()), rel, float(dB)
