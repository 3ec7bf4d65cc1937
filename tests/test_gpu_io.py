"""Output and restart on the GPU: the savedata.cpp text writer against the
oracle's state printed the same way, and checkpoint / restart continuing a
run bit for bit (FP64 and FP32, single and batched handles)."""
import os

import numpy as np
import pytest

from oracle import pyoracle as P
from parity_util import to_gpu_cfg


def cxx_default(v):
    """A double through std::ostream's default formatting (6 significant digits, %g)."""
    s = "%g" % v
    return s


@pytest.mark.gpu
def test_save4py_matches_oracle_text(gpu, tmp_path):
    kw = dict(ic="BWx", limiter="MC", flux="RUSA", cfl=0.4, maxlevs=3)
    sim = gpu.Simulation(**to_gpu_cfg(kw)).init()
    o = P.Oracle(**kw).init()
    sim.run(12)
    o.run(12)
    name = sim.save4py(str(tmp_path), id=7)
    assert os.path.basename(name).startswith("BWx007t_")
    got = open(name).read().splitlines()
    W, lp, ic, lf = o.get("W"), o.get("lp"), o.get("icoord"), o.get("leafs")
    inf = o.info()
    dx0, dy0 = inf["dx0"], inf["dy0"]
    exp = []
    hdr = "#" + "x".rjust(15) + "".join(s.rjust(16) for s in
                                        ("y", "xdelta", "ydelta", "density", "U", "v", "w", "pressure", "Bx", "By", "Bz"))
    for nb in range(inf["lastActive"]):
        if not lf[nb]:
            continue
        exp.append(hdr)
        lev = lp[nb][0]
        dx, dy = dx0 / 2 ** lev, dy0 / 2 ** lev
        for j in range(2, 18):
            y = ((j + ic[nb][1] - 2) + 0.5) * dy - dy0
            for i in range(2, 18):
                x = ((i + ic[nb][0] - 2) + 0.5) * dx - dx0
                vals = [x, y, dx / 2.0, dy / 2.0] + [W[nb, k, j, i] for k in range(8)]
                exp.append("".join(cxx_default(v).rjust(16) for v in vals))
    assert got == exp
    # full precision round-trips the state
    name17 = sim.save4py(str(tmp_path), id=8, digits=17)
    rows = np.array([list(map(float, r.split())) for r in open(name17) if not r.startswith("#")])
    leafW = np.concatenate([W[nb, :, 2:18, 2:18].reshape(8, -1).T for nb in range(inf["lastActive"]) if lf[nb]])
    assert np.array_equal(rows[:, 4:], leafW)


@pytest.mark.gpu
@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_checkpoint_restart_bitwise(gpu, tmp_path, precision):
    cfg = to_gpu_cfg(dict(ic="rotor", limiter="MC", flux="HLLD", cfl=0.4, maxlevs=4, precision=precision))
    a = gpu.Simulation(**cfg).init()
    a.run(25)
    path = str(tmp_path / "ck.bin")
    a.checkpoint_save(path)
    a.run(20)
    b = gpu.Simulation(**cfg).checkpoint_load(path)
    assert b.info()["steps"] == 25
    b.run(20)
    sa, sb = a.state(), b.state()
    assert sa["t"] == sb["t"] and sa["step"] == sb["step"]
    for k in ("lp", "icoord", "leafs", "U", "Bi"):
        assert np.array_equal(sa[k], sb[k]), k


@pytest.mark.gpu
def test_checkpoint_batch_and_errors(gpu, tmp_path):
    cfgs = [gpu.blast_config(3, i) for i in range(3)]
    for c in cfgs:
        c.maxlevs = min(c.maxlevs, 4)
    a = gpu.Simulation(cfgs).init()
    a.run(15)
    path = str(tmp_path / "ck.bin")
    a.checkpoint_save(path)
    a.run(10)
    b = gpu.Simulation(cfgs).checkpoint_load(path)
    b.run(10)
    for i in range(3):
        assert np.array_equal(a.download("U", i), b.download("U", i))
    # a different configuration or an initialised handle is refused
    other = gpu.Simulation([gpu.blast_config(4, i) for i in range(3)])
    with pytest.raises(gpu.AmrError):
        other.checkpoint_load(path)
    with pytest.raises(gpu.AmrError):
        a.checkpoint_load(path)


@pytest.mark.gpu
def test_upload_from_pinned_memory_may_be_reused_at_once(gpu):
    """amr_upload from page-locked host memory (truly asynchronous copies):
    overwriting the array right after the call must not change what the
    device received."""
    import torch
    sim = gpu.Simulation(ic="rotor", limiter="MC", flux="HLLD", cfl=0.4, maxlevs=4).init()
    sim.run(5)
    U = sim.download("U")
    pinned = torch.empty(U.shape, dtype=torch.float64, pin_memory=True)
    arr = pinned.numpy()
    arr[...] = U * 1.0001
    sim.upload("U", arr)
    arr[...] = -1.0          # the caller reuses its buffer at once
    assert np.array_equal(sim.download("U"), U * 1.0001)


@pytest.mark.gpu
def test_download_into_callers_array(gpu):
    """download(out=...) fills the caller's array when it has the field's
    shape, and allocates otherwise."""
    sim = gpu.Simulation(ic="rotor", limiter="MC", flux="HLLD", cfl=0.4, maxlevs=4).init()
    sim.run(3)
    U = sim.download("U")
    buf = np.zeros_like(U)
    got = sim.download("U", out=buf)
    assert got is buf and np.array_equal(buf, U)
    other = sim.download("U", out=np.zeros((1, 8, 20, 20)))
    assert other.shape == U.shape and np.array_equal(other, U)


@pytest.mark.gpu
def test_driver_runs_an_input_txt(gpu, tmp_path):
    """amr2d_mhd on a Brio-Wu input.txt runs to t > tEnd, writes a file every
    20 steps and one at the end (main.cpp:240-243, 262), and its step-20 file,
    written before that step's admesh, equals the library's save4py at the
    same point of the same loop."""
    import re
    import subprocess

    from amr2d_mhd_gb300 import build as B
    B.build()
    (tmp_path / "input.txt").write_text("16 16 8\n1.0 1.0 \n0.4\nBWx MC RUSA\n")
    r = subprocess.run([B.DRIVER, "--maxlevs", "3", "--quiet"], cwd=tmp_path, input="2\n0\n",
                       capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout[-2000:] + r.stderr[-2000:]
    steps = int(re.search(r"after (\d+) steps", r.stdout).group(1))
    files = sorted(os.listdir(tmp_path / "data"))
    assert steps > 40 and len(files) == steps // 20 + 1
    sim = gpu.Simulation(**to_gpu_cfg(dict(ic="BWx", limiter="MC", flux="RUSA", cfl=0.4, maxlevs=3))).init()
    sim.set_remesh(False)
    for k in range(20):
        sim.step()
        if k < 19:
            sim.admesh()
    out = tmp_path / "api"
    out.mkdir()
    name = sim.save4py(str(out), id=1)
    first = [f for f in files if f.startswith("BWx001t_")]
    assert len(first) == 1
    assert open(name).read() == open(tmp_path / "data" / first[0]).read()


@pytest.mark.gpu
@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_direct_and_staged_transfers_agree(gpu, precision):
    """Uploads and downloads through the direct path (the gather / scatter
    kernel addresses the caller's page-locked array) equal the staged copies
    (AMR2D_ZERO_COPY=0), for 16-byte aligned and unaligned arrays, pageable
    arrays and both field kinds."""
    import os
    import torch
    sims = {}
    for zc in ("1", "0"):
        os.environ["AMR2D_ZERO_COPY"] = zc
        try:
            s = gpu.Simulation(ic="rotor", limiter="MC", flux="HLLD", cfl=0.4, maxlevs=4,
                               precision=precision).init()
        finally:
            del os.environ["AMR2D_ZERO_COPY"]
        s.run(6)
        sims[zc] = s
    for field in ("U", "Bi"):
        ref = sims["0"].download(field)
        assert np.array_equal(sims["1"].download(field), ref)
        # page-locked, aligned and shifted by one double
        pin = torch.empty(ref.size + 1, dtype=torch.float64, pin_memory=True).numpy()
        for off in (0, 1):
            cur = sims["0"].download(field)
            view = pin[off:off + ref.size].reshape(ref.shape)
            got = sims["1"].download(field, out=view)
            assert np.array_equal(got, cur), (field, off)
            view[...] = cur * 1.5
            sims["1"].upload(field, view)
            sims["0"].upload(field, np.ascontiguousarray(cur * 1.5))
            assert np.array_equal(sims["1"].download(field), sims["0"].download(field)), (field, off)
        # pageable, unaligned
        raw = np.empty(ref.size + 1)
        view = raw[1:].reshape(ref.shape)
        sims["1"].download(field, out=view)
        assert np.array_equal(view, sims["0"].download(field))
    # both handles step on from the uploaded state alike
    for s in sims.values():
        s.run(3)
    assert np.array_equal(sims["1"].download("U"), sims["0"].download("U"))
