"""The oracle pinned against the reference's own answers (tests/golden/,
generated from the unmodified reference by tests/golden/make_golden.py)."""
import ast
import glob
import os

import numpy as np
import pytest

from oracle import pyoracle as P

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
import sys  # noqa: E402

sys.path.insert(0, GOLDEN)
from golden_util import leaf_hash, tree_hash  # noqa: E402

# CPU budget: long fixtures are checked on their first steps here and in
# full by the GPU tests
CPU_STEPS = 40


def test_kat_limiter():
    d = np.load(os.path.join(GOLDEN, "kat_limiter.npz"))
    got = np.array([P.slopelimiter(P.LIMITERS[li], r, e) for li, r, e in zip(d["limiter"], d["r"], d["eta"])])
    assert np.array_equal(got.view(np.int64), d["phi"].view(np.int64))


def test_kat_riemann():
    d = np.load(os.path.join(GOLDEN, "kat_riemann.npz"))
    for q in range(len(d["flux"])):
        assert d["status"][q] == 0
        got = P.riemann(P.FLUXES[d["flux"][q]], d["wL"][q], d["wR"][q], d["gamma"][q], bool(d["dir"][q]))
        assert np.array_equal(got.view(np.int64), d["out"][q].view(np.int64)), q


def test_full_state_fixture():
    d = np.load(os.path.join(GOLDEN, "state_bw_L2_mc_rusa_step10.npz"))
    meta = ast.literal_eval(str(d["meta"]))
    o = P.Oracle(ic=meta["ic"], limiter=meta["limiter"], flux=meta["flux"], cfl=meta["cfl"],
                 maxlevs=meta["maxlevs"], nghosts=meta["nghosts"]).init()
    o.run(meta["step"])
    st = o.state()
    assert st["t"] == float(d["t"])
    assert np.array_equal(st["lp"], d["lp"]) and np.array_equal(st["leafs"], d["leafs"])
    assert np.array_equal(st["U"], d["U"]) and np.array_equal(st["Bi"], d["Bi"])


RUNS = sorted(os.path.basename(p)[4:-4] for p in glob.glob(os.path.join(GOLDEN, "run_*.npz")))


@pytest.mark.parametrize("name", RUNS)
def test_run_fingerprints(name):
    d = np.load(os.path.join(GOLDEN, "run_%s.npz" % name))
    meta = ast.literal_eval(str(d["meta"]))
    o = P.Oracle(ic=meta["ic"], limiter=meta["limiter"], flux=meta["flux"], cfl=meta["cfl"],
                 maxlevs=meta["maxlevs"], nghosts=meta["nghosts"], ct_type=meta.get("ct_type", 1),
                 diffusion=meta.get("diffusion", False)).init()
    n = min(meta["steps"], CPU_STEPS)
    for s in range(n + 1):
        if s:
            o.step()
        st = o.state()
        assert st["t"] == d["t"][s] and st["dt"] == d["dt"][s], s
        assert tree_hash(st) == d["tree"][s], s
        assert leaf_hash(st) == d["leaf"][s], s


def test_kat_riemann_hydro():
    """riemannS of the reference built without a magnetic field (MAG_field =
    false, defs.hpp:32), where ROE (riemannS.cpp:297-395) runs: the oracle's
    restatement, bit for bit, every solver."""
    d = np.load(os.path.join(GOLDEN, "kat_riemann_hydro.npz"))
    assert set(d["flux"]) == {0, 1, 2, 3, 4}
    for q in range(len(d["flux"])):
        assert d["status"][q] == 0
        got = P.riemann(P.FLUXES[d["flux"][q]], d["wL"][q], d["wR"][q], d["gamma"][q], bool(d["dir"][q]),
                        mag_field=False)
        assert np.array_equal(got.view(np.int64), d["out"][q].view(np.int64)), q


LONG = sorted(os.path.basename(p)[5:-4] for p in glob.glob(os.path.join(GOLDEN, "long_*.npz")))
LONG_CPU_STEPS = 50


@pytest.mark.parametrize("name", LONG)
def test_long_run_first_steps(name):
    """The gamma-5/3 rotor of the reference (to t_end in the GPU tests): the
    oracle's first steps, t and dt each step, fingerprints where recorded."""
    d = np.load(os.path.join(GOLDEN, "long_%s.npz" % name))
    meta = ast.literal_eval(str(d["meta"]))
    o = P.Oracle(ic=meta["ic"], limiter=meta["limiter"], flux=meta["flux"], cfl=meta["cfl"],
                 maxlevs=meta["maxlevs"], nghosts=meta["nghosts"], gamma=meta["gamma"], nthreads=4).init()
    fp = {int(s): q for q, s in enumerate(d["fp_step"])}
    for s in range(LONG_CPU_STEPS + 1):
        if s:
            o.step()
        inf = o.info()
        assert inf["t"] == d["t"][s] and inf["dt"] == d["dt"][s], s
        if s in fp:
            st = o.state()
            assert tree_hash(st) == d["tree"][fp[s]], s
            assert leaf_hash(st) == d["leaf"][fp[s]], s
