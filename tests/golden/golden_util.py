"""Fingerprints of AMR states, shared by make_golden.py and the tests.

A state is the dict returned by oracle.pyoracle.read_ref_dump(),
Oracle.state() or amr2d_mhd_gb300.Simulation.state().  The leaf fingerprint
is SHA-256 over the float64 bytes of U then Bi of every leaf block in block-ID
order (layout [var][j][i], ghosts included), so two states share it only if
they are bit-identical; the tree fingerprint covers lp, icoord and leafs.
"""
import hashlib

import numpy as np


def tree_hash(st):
    na = st["lastActive"]
    h = hashlib.sha256()
    h.update(np.ascontiguousarray(st["lp"][:na], np.int32).tobytes())
    h.update(np.ascontiguousarray(st["icoord"][:na], np.int32).tobytes())
    h.update(np.ascontiguousarray(st["leafs"][:na], np.uint8).tobytes())
    return h.hexdigest()


def leaf_hash(st):
    h = hashlib.sha256()
    for b in np.nonzero(st["leafs"])[0]:
        h.update(np.ascontiguousarray(st["U"][b], np.float64).tobytes())
        h.update(np.ascontiguousarray(st["Bi"][b], np.float64).tobytes())
    return h.hexdigest()


def leaf_sums(st, ng):
    """Per-variable sum of |U| over leaf interiors (for tolerance diagnostics)."""
    lf = st["leafs"]
    return np.abs(st["U"][lf][:, :, ng:-ng, ng:-ng]).sum(axis=(0, 2, 3))


def record(st, ng):
    return dict(t=st["t"], dt=st["dt"], nleaves=int(st["leafs"].sum()), last_active=int(st["lastActive"]),
                tree=tree_hash(st), leaf=leaf_hash(st), sums=leaf_sums(st, ng))


def pack(recs):
    """records -> arrays for np.savez"""
    return dict(t=np.array([r["t"] for r in recs]), dt=np.array([r["dt"] for r in recs]),
                nleaves=np.array([r["nleaves"] for r in recs]),
                last_active=np.array([r["last_active"] for r in recs]),
                tree=np.array([r["tree"] for r in recs]), leaf=np.array([r["leaf"] for r in recs]),
                sums=np.array([r["sums"] for r in recs]))
