"""The bench's own workload pinned end to end: the MHD rotor with gamma 5/3,
5 levels, MUSCL-MC, CFL 0.4, run to t_end = 0.295.

* Reference geometry (the reference's own cells, dx0 = 1/30, meshblock.cpp:
  90-91): the FP64 CUDA path against the reference itself, built with its
  rotor's gamma set to 5/3 (IC2Dtype.cpp:77, oracle/ref.mk ROTOR_G53=1):
  t and dt of every step, and the tree and leaf-state fingerprints every 25
  steps and at the last step, bit for bit, with HLLD and with RUSA
  (tests/golden/long_rotor53_L5_mc_*.npz, tests/golden/make_golden.py).
* The bench's geometry (16 x 16 cells of 1/32 on [0,1]^2), which the
  reference cannot run: the FP64 CUDA path against the oracle to t_end, t and
  dt of every step and fingerprints every 250 steps and at the last, bit for
  bit (tests/golden/oracle_rotor53_bench_L5_mc_hlld.npz, made by the oracle,
  which the fixtures above pin to the reference), and the FP32 bulk path's
  density at t_end within 1e-4 relative L1 of FP64 on the finest uniform
  grid.
"""
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

LONG = sorted(os.path.basename(p)[5:-4] for p in glob.glob(os.path.join(GOLDEN, "long_*.npz")))
BENCH_ROTOR = dict(ic="rotor", limiter="MC", flux="HLLD", cfl=0.4, maxlevs=5, nghosts=2, geom_ref=False,
                   gamma=5.0 / 3.0)


@pytest.mark.gpu
@pytest.mark.timeout(900)
@pytest.mark.parametrize("name", LONG)
def test_gpu_long_run_matches_reference(gpu, name):
    d = np.load(os.path.join(GOLDEN, "long_%s.npz" % name))
    m = ast.literal_eval(str(d["meta"]))
    sim = gpu.Simulation(**to_gpu_cfg(dict(ic=m["ic"], limiter=m["limiter"], flux=m["flux"], cfl=m["cfl"],
                                           maxlevs=m["maxlevs"], nghosts=m["nghosts"], gamma=m["gamma"]))).init()
    fp = {int(s): q for q, s in enumerate(d["fp_step"])}
    for s in range(m["steps"] + 1):
        if s:
            sim.step()
        inf = sim.info()
        assert inf["t"] == d["t"][s] and inf["dt"] == d["dt"][s], s
        assert inf["n_leaves"] == d["nleaves"][s] and inf["last_active"] == d["last_active"][s], s
        if s in fp:
            st = sim.state()
            assert tree_hash(st) == d["tree"][fp[s]], s
            assert leaf_hash(st) == d["leaf"][fp[s]], s
    assert sim.info()["done"] == 1          # the reference's last step is ours
    assert m["steps"] in fp


@pytest.mark.gpu
@pytest.mark.timeout(900)
def test_gpu_bench_rotor_to_t_end(gpu):
    d = np.load(os.path.join(GOLDEN, "oracle_rotor53_bench_L5_mc_hlld.npz"))
    m = ast.literal_eval(str(d["meta"]))
    cfg = to_gpu_cfg(BENCH_ROTOR)
    a = gpu.Simulation(**cfg).init()
    fp = {int(s): q for q, s in enumerate(d["fp_step"])}
    for s in range(m["steps"] + 1):
        if s:
            a.step()
        inf = a.info()
        assert inf["t"] == d["t"][s] and inf["dt"] == d["dt"][s], s
        assert inf["n_leaves"] == d["nleaves"][s], s
        if s in fp:
            st = a.state()
            assert tree_hash(st) == d["tree"][fp[s]], s
            assert leaf_hash(st) == d["leaf"][fp[s]], s
    assert a.info()["done"] == 1 and a.info()["t"] > 0.295
    b = gpu.Simulation(**dict(cfg, precision="fp32")).init()
    b.run()
    assert b.info()["t"] > 0.295
    r64, r32 = a.uniform(0), b.uniform(0)
    l1 = float(np.abs(r32 - r64).sum() / np.abs(r64).sum())
    print("rotor t_end FP32 vs FP64 density relative L1: %.3e" % l1)
    assert l1 <= 1e-4, l1
