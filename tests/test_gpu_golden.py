"""The FP64 CUDA path against the reference's own per-step fingerprints
(tests/golden/run_*.npz), over the full length of every fixture, including
the complete Brio-Wu run to t = 0.2 (453 steps, 4 levels)."""
import ast
import glob
import os
import sys

import numpy as np
import pytest

from parity_util import to_gpu_cfg

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
sys.path.insert(0, GOLDEN)
from golden_util import leaf_hash, tree_hash  # noqa: E402

RUNS = sorted(os.path.basename(p)[4:-4] for p in glob.glob(os.path.join(GOLDEN, "run_*.npz")))


@pytest.mark.gpu
@pytest.mark.parametrize("name", RUNS)
def test_gpu_run_fingerprints(gpu, name):
    d = np.load(os.path.join(GOLDEN, "run_%s.npz" % name))
    m = ast.literal_eval(str(d["meta"]))
    sim = gpu.Simulation(**to_gpu_cfg(dict(ic=m["ic"], limiter=m["limiter"], flux=m["flux"], cfl=m["cfl"],
                                           maxlevs=m["maxlevs"], nghosts=m["nghosts"],
                                           ct_type=m.get("ct_type", 1), diffusion=m.get("diffusion", False)))).init()
    for s in range(m["steps"] + 1):
        if s:
            sim.step()
        inf = sim.info()
        assert inf["t"] == d["t"][s] and inf["dt"] == d["dt"][s], s
        assert inf["n_leaves"] == d["nleaves"][s], s
        if s % 10 == 0 or s == m["steps"]:
            st = sim.state()
            assert tree_hash(st) == d["tree"][s], s
            assert leaf_hash(st) == d["leaf"][s], s
    if name.endswith("_full"):
        assert sim.info()["done"] == 1


@pytest.mark.gpu
def test_gpu_full_state_fixture(gpu):
    d = np.load(os.path.join(GOLDEN, "state_bw_L2_mc_rusa_step10.npz"))
    m = ast.literal_eval(str(d["meta"]))
    sim = gpu.Simulation(**to_gpu_cfg(dict(ic=m["ic"], limiter=m["limiter"], flux=m["flux"], cfl=m["cfl"],
                                           maxlevs=m["maxlevs"], nghosts=m["nghosts"]))).init()
    sim.run(m["step"])
    st = sim.state()
    assert np.array_equal(st["lp"], d["lp"]) and np.array_equal(st["leafs"], d["leafs"])
    assert np.array_equal(st["U"], d["U"]) and np.array_equal(st["Bi"], d["Bi"])
