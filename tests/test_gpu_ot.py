"""Orszag-Tang (extension IC) on the GPU: FP32 bulk path against the FP64
path on a common fixed time grid to t = pi, relative L1 per conserved
variable on the finest uniform grid.  (FP64 against the oracle: the OT cases
of test_gpu_parity.py.)"""
import numpy as np
import pytest


def run(gpu, ml, lim, dt, precision):
    sim = gpu.Simulation(gpu.ot_config(ml, precision, limiter=lim, dt_fixed=dt)).init()
    sim.run()
    inf = sim.info()
    assert inf["done"] and abs(inf["t"] - np.pi) < 2 * dt
    return [sim.uniform(k) for k in range(8)]


@pytest.mark.gpu
@pytest.mark.parametrize("ml,lim,dt,tol", [(3, "WENO5", 0.003, 5e-3), (4, "MC", 0.0015, 1e-4)])
def test_ot_fp32_close_to_fp64(gpu, ml, lim, dt, tol):
    a = run(gpu, ml, lim, dt, "fp64")
    b = run(gpu, ml, lim, dt, "fp32")
    for k in (0, 1, 2, 4, 5, 6):
        l1 = np.abs(b[k] - a[k]).sum() / np.abs(a[k]).sum()
        assert l1 < tol, (k, l1)
    assert np.abs(a[3]).max() == 0.0 and np.abs(a[7]).max() == 0.0   # 2-D flow: no z components
