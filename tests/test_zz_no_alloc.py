"""amr_cfl_dt_static, the CFL reduction for callers that cannot allocate.

Hosts that may not call cudaMalloc when they need the time step -- code
inside a captured CUDA graph, allocator-free real-time loops, frameworks that
own every device allocation -- call amr_cfl_dt_static with their own device
arrays; its per-block scratch is a fixed 65536-entry array in the library's
device globals.  The test checks it through the C ABI against amr_cfl_dt, on
two calls in a row, with 2 ghost layers (MUSCL) and 4 (WENO5).  This file
sorts last so that a run that stops at the first failure has already run
every other test.
"""
import ctypes

import numpy as np
import pytest


def _dxdy(lp, lf, lenx=1.0, nroots=2, ni=16):
    dx0 = lenx / (float(nroots) * (ni - 1))   # meshblock.cpp:90, reference geometry
    out = []
    for b in np.nonzero(lf)[0]:
        d = dx0
        for _ in range(int(lp[b, 0])):
            d = d / 2.0
        out.append((d, d))
    return np.array(out, np.float64)


@pytest.mark.gpu
@pytest.mark.parametrize("limiter,nghosts,maxlevs", [("MC", 2, 4), ("WENO5", 4, 3)])
def test_cfl_dt_static_matches_cfl_dt(gpu, limiter, nghosts, maxlevs):
    import torch

    L = gpu.load()
    sim = gpu.Simulation(ic="rotor", limiter=limiter, flux="HLLD", cfl=0.4, maxlevs=maxlevs,
                         nghosts=nghosts).init()
    stream = torch.cuda.current_stream()
    out = torch.empty(1, dtype=torch.float64, device="cuda")
    for call in range(2):
        sim.run(25)
        expect = sim.cfl_dt()
        lp, _, lf = sim.tree()
        U = torch.from_numpy(np.ascontiguousarray(sim.download("U")[lf])).cuda()
        dxdy = torch.from_numpy(_dxdy(lp, lf)).cuda()
        torch.cuda.synchronize()
        free0 = torch.cuda.mem_get_info()[0]
        rc = L.amr_cfl_dt_static(ctypes.c_void_p(U.data_ptr()), int(lf.sum()), nghosts,
                                 ctypes.c_void_p(dxdy.data_ptr()), sim.info()["gamma"],
                                 ctypes.c_void_p(out.data_ptr()), ctypes.c_void_p(stream.cuda_stream))
        assert rc == 0
        torch.cuda.synchronize()
        got = out.item()
        # FP64 parity tolerance of this suite: bit-identical
        assert got == expect, (call, got, expect)
        if call == 1:   # the first call loads the module; later calls allocate nothing
            assert torch.cuda.mem_get_info()[0] == free0


@pytest.mark.gpu
def test_cfl_dt_static_rejects_too_many_blocks(gpu):
    import torch

    L = gpu.load()
    x = torch.zeros(8, dtype=torch.float64, device="cuda")
    rc = L.amr_cfl_dt_static(ctypes.c_void_p(x.data_ptr()), 65537, 2, ctypes.c_void_p(x.data_ptr()), 1.4,
                             ctypes.c_void_p(x.data_ptr()), None)
    assert rc == -13
