"""The product's host code (no GPU needed): the compiled ghost fills and the
quadtree's admesh, against the oracle's sequential restatement."""
import numpy as np
import pytest

from oracle import pyoracle as P
from shim import admesh, ghost_apply, host_pool

GHOST_CASES = [("BWx", "MC", 4, 2, 3), ("rotor", "MC", 5, 2, 30), ("BWx", "WENO5", 3, 4, 10),
               ("rotor", "WENO5", 3, 4, 25)]


@pytest.mark.parametrize("ic,lim,L,ng,steps", GHOST_CASES)
def test_ghost_program_matches_sequential_fill(ic, lim, L, ng, steps):
    o = P.Oracle(ic=ic, limiter=lim, flux="RUSA", cfl=0.4, maxlevs=L, nghosts=ng).init()
    for _ in range(steps):
        o.step()
    st = o.state()
    n = 16 + 2 * ng
    rng = np.random.default_rng(steps)
    for kind, nv in [(0, 8), (1, 2), (1, 8), (2, 1)]:
        f = rng.standard_normal((st["lastActive"], nv, n, n))
        ref = o.fill(f, kind)
        got, nops, _ = ghost_apply(st, kind, nv, f, L, ng)
        assert nops > 0
        assert np.array_equal(ref, got), (kind, nv, int((ref != got).sum()))


def test_ghost_program_periodic_16_roots():
    o = P.Oracle(ic="OT", limiter="MC", flux="RUSA", cfl=0.4, maxlevs=3, nroots=(4, 4), periodic=True,
                 geom_ref=False, lenx=2 * np.pi, leny=2 * np.pi).init()
    for _ in range(3):
        o.step()
    st = o.state()
    f = np.random.default_rng(1).standard_normal((st["lastActive"], 8, 20, 20))
    got, _, _ = ghost_apply(st, 0, 8, f, 3, 2, (4, 4), True)
    assert np.array_equal(o.fill(f, 0), got)


@pytest.mark.parametrize("ic,flux,L,steps", [("rotor", "RUSA", 5, 40), ("BWx", "RUSA", 4, 12)])
def test_admesh_matches_oracle(ic, flux, L, steps):
    o = P.Oracle(ic=ic, limiter="MC", flux=flux, cfl=0.4, maxlevs=L).init()
    o.set_remesh(False)
    changes = 0
    for _ in range(steps):
        o.step()
        st = o.state()
        grad = P.criteria_grad(o.get("W"))
        got, nr, nc = admesh(st, grad, L)
        o.admesh()
        ref = o.state()
        changes += nr + nc
        assert got["lastActive"] == ref["lastActive"]
        assert np.array_equal(got["leafs"], ref["leafs"])
        assert np.array_equal(got["lp"], ref["lp"])
        assert np.array_equal(got["icoord"], ref["icoord"])
        assert got["nbleafs"] == ref["nbleafs"]
    assert changes > 0


@pytest.mark.parametrize("threads", [1, 2, 8])
def test_host_pool_parallel_loops(threads):
    """The engine's persistent host threads (remesh, compile and layout loops
    of a batch): 300 consecutive loops of 1000 items, every item once."""
    assert host_pool(300, 1000, threads) == 0
