"""Fused ghost fills: the step with every fill gathered inside the kernel that
consumes the field (and its snapshots saved by the kernel before) leaves the
state bit-identical to the step with each fill as launches of its own
(AMR2D_FUSED_FILLS=0), in both precisions, both stage kernels, batches, the
upwind CT EMF, diffusion and four ghost layers; and it launches fewer
kernels per step."""
import os

import numpy as np
import pytest

from parity_util import to_gpu_cfg

CASES = {
    "rotor_hlld_split": (dict(ic="rotor", limiter="MC", flux="HLLD", cfl=0.4, maxlevs=5), "split", 40),
    "rotor_hlld_fused": (dict(ic="rotor", limiter="MC", flux="HLLD", cfl=0.4, maxlevs=5), "fused", 40),
    "rotor_fp32": (dict(ic="rotor", limiter="MC", flux="HLLD", cfl=0.4, maxlevs=5, precision="fp32"), "fused", 40),
    "bwy_weno5_hllc": (dict(ic="BWy", limiter="WENO5", flux="HLLC", cfl=0.4, maxlevs=4, nghosts=4), "split", 25),
    "rotor_ct2_diff": (dict(ic="rotor", limiter="VanLeer", flux="HLLE", cfl=0.4, maxlevs=5, ct_type=2,
                            diffusion=True), "fused", 30),
    "ot_periodic": (dict(ic="OT", limiter="MC", flux="HLLD", cfl=0.4, maxlevs=4, nroots=(3, 3), periodic=True,
                         geom_ref=False, lenx=2 * np.pi, leny=2 * np.pi), "split", 25),
    "bwx_weno5_fp32_fused": (dict(ic="BWx", limiter="WENO5", flux="HLLD", cfl=0.4, maxlevs=4, nghosts=4,
                                  precision="fp32"), "fused", 25),
}


def make(gpu, configs, kernel, fused, coop=True, graphs=True):
    env = {"AMR2D_STAGE_KERNEL": kernel, "AMR2D_FUSED_FILLS": "1" if fused else "0",
           "AMR2D_CT_COOP": "1" if coop else "0", "AMR2D_GRAPHS": "1" if graphs else "0"}
    old = {k: os.environ.get(k) for k in env}
    os.environ.update(env)
    try:
        if isinstance(configs, dict):
            return gpu.Simulation(**to_gpu_cfg(configs)).init()
        return gpu.Simulation(configs).init()
    finally:
        for k, v in old.items():
            if v is None:
                del os.environ[k]
            else:
                os.environ[k] = v


def launches_per_step(sim, steps):
    sim.profile(True)
    sim.run(steps)
    p = sim.profile()
    sim.profile(False)
    return p["launches"] / max(p["steps"], 1)


def same_state(a, b, n):
    for i in range(n):
        sa, sb = a.state(i), b.state(i)
        assert sa["t"] == sb["t"] and sa["dt"] == sb["dt"], i
        assert np.array_equal(sa["lp"], sb["lp"]) and np.array_equal(sa["leafs"], sb["leafs"]), i
        assert np.array_equal(sa["U"], sb["U"]), (i, int((sa["U"] != sb["U"]).sum()))
        assert np.array_equal(sa["Bi"], sb["Bi"]), i


@pytest.mark.gpu
@pytest.mark.parametrize("coop", [True, False], ids=["ct_coop", "ct_3"])
@pytest.mark.parametrize("case", sorted(CASES))
def test_fused_fills_bit_identical(gpu, case, coop):
    """coop: the three CT kernels of a stage as one cooperative launch with
    grid barriers (6 launches per step with the fused stage kernel)."""
    cfg, kernel, steps = CASES[case]
    a = make(gpu, cfg, kernel, True, coop)
    b = make(gpu, cfg, kernel, False)
    la = launches_per_step(a, steps)
    lb = launches_per_step(b, steps)
    same_state(a, b, 1)
    print("%s %s: %.1f launches per step fused, %.1f unfused" % (case, "coop" if coop else "3 CT", la, lb))
    assert la < lb
    if coop and kernel == "fused":
        assert la <= 8


@pytest.mark.gpu
@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_fused_fills_blast_batch(gpu, precision):
    """Uneven seeded blast instances in one handle (instances finish at
    different times, so the program's layout changes under the fused fills)."""
    cfgs = []
    for i in range(5):
        c = gpu.blast_config(20261204, i, precision)
        c.maxlevs = min(c.maxlevs, 4)
        c.t_end = 0.004 * (i + 1)
        cfgs.append(c)
    # each stage kernel against itself: the FP32 split and fused stage
    # kernels round differently (FMA contraction in the fused one)
    a = make(gpu, cfgs, "fused", True)
    b = make(gpu, cfgs, "fused", False)
    c = make(gpu, cfgs, "split", True)
    d = make(gpu, cfgs, "split", False)
    for _ in range(4):
        for sim in (a, b, c, d):
            sim.run(12)
        same_state(a, b, len(cfgs))
        same_state(c, d, len(cfgs))


@pytest.mark.gpu
@pytest.mark.parametrize("kernel", ["fused", "split"])
def test_fused_fills_without_graphs(gpu, kernel):
    """The fused step launched kernel by kernel (no captured graph) equals the
    captured one, and the separate fills."""
    cfg = dict(ic="rotor", limiter="MC", flux="HLLD", cfl=0.4, maxlevs=5)
    a = make(gpu, cfg, kernel, True, graphs=False)
    b = make(gpu, cfg, kernel, True)
    c = make(gpu, cfg, kernel, False)
    for sim in (a, b, c):
        sim.run(30)
    same_state(a, b, 1)
    same_state(a, c, 1)
