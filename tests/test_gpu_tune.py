"""Launch schedules: the autotuner's choice, and each stage schedule, leave
the FP64 path bit-identical to the oracle."""
import os

import numpy as np
import pytest

from oracle import pyoracle as P
from parity_util import to_gpu_cfg

KW = dict(ic="rotor", limiter="MC", flux="HLLD", cfl=0.4, maxlevs=4)


def same_as_oracle(sim, o):
    a, b = sim.state(), o.state()
    same, dU, rel, dB = P.compare_states(a, b, 2)
    return same and np.array_equal(a["U"], b["U"]) and np.array_equal(a["Bi"], b["Bi"]) and a["t"] == b["t"]


@pytest.mark.gpu
def test_autotune_keeps_parity(gpu):
    sim = gpu.Simulation(**to_gpu_cfg(KW)).init()
    o = P.Oracle(**KW).init()
    sim.run(10)
    report = sim.autotune(2)
    lines = report.strip().splitlines()
    assert len(lines) == 42 and sum(l.startswith("*") for l in lines) == 1
    sim.run(20)
    o.run(30)
    assert same_as_oracle(sim, o)


@pytest.mark.gpu
@pytest.mark.parametrize("kernel", ["fused", "split"])
def test_stage_schedules_parity(gpu, kernel):
    os.environ["AMR2D_STAGE_KERNEL"] = kernel
    try:
        sim = gpu.Simulation(**to_gpu_cfg(KW)).init()
    finally:
        del os.environ["AMR2D_STAGE_KERNEL"]
    o = P.Oracle(**KW).init()
    sim.run(25)
    o.run(25)
    assert same_as_oracle(sim, o)
