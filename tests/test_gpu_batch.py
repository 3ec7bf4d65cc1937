"""Batches of independent problems on the GPU: the seeded blast batch against
the oracle instance by instance, FP32 against FP64, and the fixed-dt
Kelvin-Helmholtz problem."""
import numpy as np
import pytest

from oracle import pyoracle as P
from parity_util import oracle_kw


def blast_batch(gpu, seed, n, cap_levels, precision="fp64", t_end=None):
    cfgs = []
    for i in range(n):
        c = gpu.blast_config(seed, i, precision)
        c.maxlevs = min(c.maxlevs, cap_levels)
        if t_end is not None:
            c.t_end = t_end
        cfgs.append(c)
    return cfgs


@pytest.mark.gpu
def test_blast_batch_matches_oracle(gpu):
    """Six seeded blast instances of uneven size in one handle reproduce the
    oracle bit for bit, tree and state, instance by instance."""
    cfgs = blast_batch(gpu, 20261203, 6, 4)
    sim = gpu.Simulation(cfgs).init()
    orc = [P.Oracle(**oracle_kw(c)).init() for c in cfgs]
    for _ in range(3):
        sim.run(15)
        leaves = []
        for i, o in enumerate(orc):
            o.run(o.info()["count"] + 15)
            a, b = sim.state(i), o.state()
            same, dU, rel, dB = P.compare_states(a, b, 2)
            assert same, i
            assert np.array_equal(a["U"], b["U"]) and np.array_equal(a["Bi"], b["Bi"]), (i, dU, dB)
            assert a["t"] == b["t"]
            leaves.append(int(b["leafs"].sum()))
    assert len(set(leaves)) > 1  # uneven instances


@pytest.mark.gpu
def test_batch_mixed_ct_and_diffusion_matches_oracle(gpu):
    """Rotor instances with the basic and the upwind CT EMF, with and without
    diffusion, in one handle: each reproduces the oracle bit for bit."""
    opts = [dict(), dict(ct_type=2), dict(diffusion=True), dict(ct_type=2, diffusion=True)]
    cfgs = [gpu.make_config(ic="rotor", limiter="MC", flux="HLLD", cfl=0.4, maxlevs=4, **o) for o in opts]
    sim = gpu.Simulation(cfgs).init()
    orc = [P.Oracle(**oracle_kw(c)).init() for c in cfgs]
    sim.run(30)
    states = []
    for i, o in enumerate(orc):
        o.run(30)
        a, b = sim.state(i), o.state()
        assert P.compare_states(a, b, 2)[0], i
        assert np.array_equal(a["U"], b["U"]) and np.array_equal(a["Bi"], b["Bi"]), i
        states.append(a)
    # the options change the solution
    assert not np.array_equal(states[0]["U"], states[1]["U"]) and not np.array_equal(states[0]["U"], states[2]["U"])


@pytest.mark.gpu
def test_ct2_diffusion_fp32_close_to_fp64(gpu):
    """FP32 bulk path with the upwind CT EMF and diffusion: rotor (4 levels)
    to t = 0.05 against FP64, relative L1 density on the finest grid."""
    kw = dict(ic="rotor", limiter="MC", flux="HLLD", cfl=0.4, maxlevs=4, ct_type=2, diffusion=True, t_end=0.05)
    a = gpu.Simulation(**kw).init()
    b = gpu.Simulation(precision="fp32", **kw).init()
    a.run()
    b.run()
    r64, r32 = a.uniform(0), b.uniform(0)
    l1 = np.abs(r32 - r64).sum() / np.abs(r64).sum()
    assert l1 < 1e-3, l1


@pytest.mark.gpu
def test_split_step_pipelines_two_handles(gpu):
    """Eight blast instances in one handle against the same eight split over
    two handles (each on its own stream) stepped with amr_step_begin /
    amr_step_end interleaved: every instance ends bit-identical."""
    cfgs = blast_batch(gpu, 7, 8, 4)
    one = gpu.Simulation(cfgs).init()
    a, b = gpu.Simulation(cfgs[:4]).init(), gpu.Simulation(cfgs[4:]).init()
    one.run(25)
    a.step_begin()
    for k in range(25):
        b.step_begin()
        a.step_end()
        if k + 1 < 25:
            a.step_begin()
        b.step_end()
    assert a.info(0)["steps"] == 25 and b.info(3)["steps"] == 25
    for i in range(8):
        s, q = (a, i) if i < 4 else (b, i - 4)
        x, y = one.state(i), s.state(q)
        assert P.compare_states(x, y, 2)[0], i
        assert np.array_equal(x["U"], y["U"]) and np.array_equal(x["Bi"], y["Bi"]) and x["t"] == y["t"], i
    # a call on a handle with a step in flight finishes that step first
    a.step_begin()
    assert a.info(0)["steps"] == 26
    a.step_end()   # nothing in flight: no-op
    assert a.info(0)["steps"] == 26


@pytest.mark.gpu
def test_blast_batch_fp32_close_to_fp64(gpu):
    """Four blast instances (4 levels at most) run to t = 0.1 in FP32 and in
    FP64; relative L1 density difference on the finest uniform grid."""
    a = gpu.Simulation(blast_batch(gpu, 99, 4, 4)).init()
    b = gpu.Simulation(blast_batch(gpu, 99, 4, 4, "fp32")).init()
    a.run()
    b.run()
    for i in range(4):
        assert a.info(i)["done"] and b.info(i)["done"]
        r64, r32 = a.uniform(0, instance=i), b.uniform(0, instance=i)
        l1 = np.abs(r32 - r64).sum() / np.abs(r64).sum()
        assert l1 < 1e-3, (i, l1)


@pytest.mark.gpu
def test_kh_fixed_dt_matches_oracle(gpu):
    """Frozen 256^2 periodic Kelvin-Helmholtz layer with dt fixed at 2e-4."""
    c = gpu.kh_config(5)
    sim = gpu.Simulation(c).init()
    o = P.Oracle(**oracle_kw(c, 16)).init()
    sim.run(12)
    o.run(12)
    a, b = sim.state(), o.state()
    assert np.array_equal(a["U"], b["U"]) and np.array_equal(a["Bi"], b["Bi"])
    assert a["t"] == b["t"] and abs(a["t"] - 12 * 2e-4) < 1e-15
    assert a["dt"] == 2e-4
