"""CPU shim over the product's host code (ghost-fill compiler and quadtree):
tests/ghost_shim.cpp compiled together with amr2d_mhd_gb300/csrc/{ghost_compile,tree}.cpp."""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)
CSRC = os.path.join(REPO, "amr2d_mhd_gb300", "csrc")
OUT = os.path.join(HERE, "_build", "ghost_shim.so")
_lib = None


def lib():
    global _lib
    if _lib is None:
        srcs = [os.path.join(HERE, "ghost_shim.cpp"), os.path.join(CSRC, "ghost_compile.cpp"),
                os.path.join(CSRC, "tree.cpp")]
        deps = srcs + [os.path.join(CSRC, f) for f in ("ghost_compile.hpp", "tree.hpp", "amr_common.h")]
        if not os.path.exists(OUT) or os.path.getmtime(OUT) < max(os.path.getmtime(d) for d in deps):
            os.makedirs(os.path.dirname(OUT), exist_ok=True)
            tmp = OUT + ".%d" % os.getpid()
            subprocess.check_call(["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-fPIC", "-shared",
                                   "-I" + CSRC] + srcs + ["-o", tmp])
            os.replace(tmp, OUT)
        L = ctypes.CDLL(OUT)
        L.ghost_shim_apply.argtypes = [ctypes.c_int] + [ctypes.c_void_p] * 3 + [ctypes.c_int] * 7 + \
            [ctypes.c_void_p] * 3
        L.tree_shim_admesh.argtypes = [ctypes.c_void_p] * 5 + [ctypes.c_int] * 5 + [ctypes.c_void_p, ctypes.c_int] + \
            [ctypes.c_void_p] * 4
        L.ghost_shim_last_by_block.argtypes = []
        L.ghost_shim_apply_fused.argtypes = [ctypes.c_int] + [ctypes.c_void_p] * 3 + [ctypes.c_int] * 7 + \
            [ctypes.c_void_p, ctypes.c_uint]
        L.host_pool_shim.argtypes = [ctypes.c_int] * 3
        L.tree_shim_check.argtypes = [ctypes.c_int] + [ctypes.c_void_p] * 3 + [ctypes.c_int] * 5 + \
            [ctypes.c_char_p, ctypes.c_int]
        _lib = L
    return _lib


def ghost_apply(st, kind, nv, field, maxlevs, ng=2, nroots=(2, 2), periodic=False):
    a = np.array(field, dtype=np.float64, copy=True)
    lp = np.ascontiguousarray(st["lp"], np.int32)
    ic = np.ascontiguousarray(st["icoord"], np.int32)
    lf = np.ascontiguousarray(st["leafs"].astype(np.uint8))
    no, ns = ctypes.c_int(), ctypes.c_int()
    rc = lib().ghost_shim_apply(st["lastActive"], lp.ctypes.data, ic.ctypes.data, lf.ctypes.data, maxlevs,
                                nroots[0], nroots[1], int(periodic), ng, kind, nv, a.ctypes.data,
                                ctypes.byref(no), ctypes.byref(ns))
    assert rc == 0
    return a, no.value, ns.value


def ghost_apply_fused(st, kind, nv, field, maxlevs, seed, ng=2, nroots=(2, 2), periodic=False):
    """The compiled fill applied block by block in a shuffled order, in place
    (as the fused kernels apply it), after every block's snapshots."""
    a = np.array(field, dtype=np.float64, copy=True)
    lp = np.ascontiguousarray(st["lp"], np.int32)
    ic = np.ascontiguousarray(st["icoord"], np.int32)
    lf = np.ascontiguousarray(st["leafs"].astype(np.uint8))
    rc = lib().ghost_shim_apply_fused(st["lastActive"], lp.ctypes.data, ic.ctypes.data, lf.ctypes.data, maxlevs,
                                      nroots[0], nroots[1], int(periodic), ng, kind, nv, a.ctypes.data, seed)
    assert rc == 0, rc
    return a


def last_by_block():
    """1 if the program of the last ghost_apply call had every written and
    every saved cell in a leaf block (the fused fills' condition)."""
    return lib().ghost_shim_last_by_block()


def admesh(st, grad, maxlevs, ng=2, nroots=(2, 2), periodic=False, cap=100000, marks=None):
    """Tree::admesh on the criterion `grad`, or Tree::admesh_marked on
    marks = (iref, icoarse) when grad is None."""
    na = ctypes.c_int(st["lastActive"])
    nbl = ctypes.c_int(st["nbleafs"])
    lp = np.zeros((cap, 8), np.int32)
    ic = np.zeros((cap, 2), np.int32)
    lf = np.zeros(cap, np.uint8)
    n0 = st["lastActive"]
    lp[:n0], ic[:n0], lf[:n0] = st["lp"], st["icoord"], st["leafs"]
    g = None if grad is None else np.ascontiguousarray(grad, np.float64)
    mr = mc = None
    if marks is not None:
        mr = np.ascontiguousarray(marks[0], np.uint8)
        mc = np.ascontiguousarray(marks[1], np.uint8)
        assert mr.size >= n0 and mc.size >= n0
    nr, nc = ctypes.c_int(), ctypes.c_int()
    rc = lib().tree_shim_admesh(ctypes.byref(na), lp.ctypes.data, ic.ctypes.data, lf.ctypes.data, ctypes.byref(nbl),
                                maxlevs, nroots[0], nroots[1], int(periodic), ng,
                                None if g is None else g.ctypes.data, cap, ctypes.byref(nr), ctypes.byref(nc),
                                None if mr is None else mr.ctypes.data, None if mc is None else mc.ctypes.data)
    assert rc == 0, rc
    n = na.value
    return dict(lastActive=n, nbleafs=nbl.value, lp=lp[:n], icoord=ic[:n], leafs=lf[:n].astype(bool)), nr.value, nc.value


def tree_check(st, maxlevs, ng=2, nroots=(2, 2), periodic=False):
    """Tree::check: None when the tree passes, else the message."""
    lp = np.ascontiguousarray(st["lp"], np.int32)
    ic = np.ascontiguousarray(st["icoord"], np.int32)
    lf = np.ascontiguousarray(np.asarray(st["leafs"]).astype(np.uint8))
    buf = ctypes.create_string_buffer(256)
    rc = lib().tree_shim_check(st["lastActive"], lp.ctypes.data, ic.ctypes.data, lf.ctypes.data, maxlevs,
                               nroots[0], nroots[1], int(periodic), ng, buf, 256)
    assert rc in (0, 1), rc
    return None if rc == 0 else buf.value.decode()


def host_pool(rounds, n, threads):
    return lib().host_pool_shim(rounds, n, threads)
