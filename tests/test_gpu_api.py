"""C-ABI behaviour on the GPU: the reference-function entry points, state
exchange, error reporting, batches and the FP32 path."""
import numpy as np
import pytest

from oracle import pyoracle as P
from parity_util import to_gpu_cfg


@pytest.mark.gpu
def test_individual_calls_reproduce_one_step(gpu):
    """main.cpp:128-246 issued call by call equals amr_step (first step, dt = 0)."""
    kw = to_gpu_cfg(dict(ic="BWx", limiter="MC", flux="RUSA", cfl=0.4, maxlevs=3))
    a = gpu.Simulation(**kw).init()
    b = gpu.Simulation(**kw).init()
    a.step()
    b.locate_bounds()
    b.boundary("U")
    b.boundary("Bi")
    b.MUSCL2D(1)
    b.boundary("Bi")
    b.boundary("ff")
    b.boundary("gg")
    b.CT2D(1)
    b.boundary("Us")
    b.MUSCL2D(2)
    b.boundary("ff")
    b.boundary("gg")
    b.CT2D(2)
    b.boundary("U")
    lam = b.cfl_dt()
    assert lam > 0
    b.admesh()
    assert np.array_equal(a.tree()[0], b.tree()[0])
    for f in ("U", "Bi", "Us", "Bis"):
        assert np.array_equal(a.download(f), b.download(f)), f


@pytest.mark.gpu
def test_upload_download_roundtrip(gpu):
    sim = gpu.Simulation(**to_gpu_cfg(dict(ic="rotor", limiter="MC", flux="RUSA", maxlevs=3))).init()
    sim.run(3)
    U = sim.download("U")
    B = sim.download("Bi")
    rng = np.random.default_rng(0)
    X = rng.standard_normal(U.shape)
    sim.upload("U", X)
    assert np.array_equal(sim.download("U"), X)
    sim.upload("U", U)
    sim.upload("Bi", B)
    W = sim.download("W")
    o = P.Oracle(ic="rotor", limiter="MC", flux="RUSA", cfl=0.4, maxlevs=3).init()
    o.run(3)
    assert np.allclose(W[o.get("leafs")], o.get("W")[o.get("leafs")], rtol=0, atol=0)


@pytest.mark.gpu
def test_negative_pressure_is_reported(gpu):
    """meshblock.cpp:136-142: a non-positive interior pressure stops the run
    with AMR_E_PRESSURE (the state is prepared on the host)."""
    sim = gpu.Simulation(**to_gpu_cfg(dict(ic="BWx", limiter="MC", flux="RUSA", maxlevs=2))).init()
    U = sim.download("U")
    lp, ic, lf = sim.tree()
    b = int(np.nonzero(lf)[0][0])
    U[b, 4, 8, 8] = 0.5 * (U[b, 1, 8, 8] ** 2 + U[b, 2, 8, 8] ** 2) / U[b, 0, 8, 8] - 1.0  # E below kinetic+magnetic
    sim.upload("U", U)
    with pytest.raises(gpu.AmrError) as e:
        sim.step()
    assert e.value.code == -5
    with pytest.raises(gpu.AmrError) as e:   # the handle stays stopped
        sim.step()
    assert e.value.code == -9


@pytest.mark.gpu
def test_step_before_init(gpu):
    sim = gpu.Simulation(**to_gpu_cfg(dict(ic="BWx", maxlevs=2)))
    with pytest.raises(gpu.AmrError) as e:
        sim.step()
    assert e.value.code == -9


@pytest.mark.gpu
def test_batch_matches_single_instances(gpu):
    """A batch sweeps independent problems in the same launches; each instance
    is bit-identical to running it alone."""
    cfgs = [dict(ic="BWx", maxlevs=3), dict(ic="rotor", maxlevs=4), dict(ic="SSTy", limiter="MC", maxlevs=2)]
    full = [to_gpu_cfg(dict(flux="RUSA", cfl=0.4, **c)) for c in cfgs]
    batch = gpu.Simulation([gpu.make_config(**c) for c in full]).init()
    singles = [gpu.Simulation(**c).init() for c in full]
    for _ in range(15):
        batch.step()
        for s in singles:
            s.step()
    for q, s in enumerate(singles):
        assert batch.info(q)["t"] == s.info()["t"]
        assert np.array_equal(batch.download("U", q), s.download("U"))
        assert np.array_equal(batch.download("Bi", q), s.download("Bi"))


@pytest.mark.gpu
def test_fp32_density_close_to_fp64(gpu):
    """FP32 bulk vs the FP64 path on the rotor after 200 steps: relative L1
    density error on leaf interiors (same tree required for the comparison)."""
    kw = to_gpu_cfg(dict(ic="rotor", limiter="MC", flux="HLLD", cfl=0.4, maxlevs=4))
    a = gpu.Simulation(**kw).init()
    kw["precision"] = "fp32"
    b = gpu.Simulation(**kw).init()
    a.run(200)
    b.run(200)
    sa, sb = a.state(), b.state()
    assert np.array_equal(sa["leafs"], sb["leafs"])
    lf = sa["leafs"]
    ra, rb = sa["U"][lf][:, 0, 2:-2, 2:-2], sb["U"][lf][:, 0, 2:-2, 2:-2]
    err = np.abs(ra - rb).sum() / np.abs(ra).sum()
    assert err < 1e-4, err


@pytest.mark.gpu
def test_criteria_matches_oracle(gpu):
    """amr_criteria (device reduction) equals criteria.cpp evaluated by the
    oracle's helper on the same state, bit for bit."""
    kw = dict(ic="rotor", limiter="MC", flux="HLLD", cfl=0.4, maxlevs=4)
    sim = gpu.Simulation(**to_gpu_cfg(kw)).init()
    o = P.Oracle(**kw).init()
    sim.run(12)
    o.run(12)
    g = sim.criteria()
    lf = o.get("leafs")
    U = o.get("U")
    gm = o.info()["gamma"] - 1
    W = U.copy()
    W[:, 1:4] = U[:, 1:4] / U[:, :1]
    p = gm * (U[:, 4] - 0.5 * U[:, 0] * (W[:, 1] * W[:, 1] + W[:, 2] * W[:, 2] + W[:, 3] * W[:, 3]))
    W[:, 4] = p - gm * (0.5 * (U[:, 5] * U[:, 5] + U[:, 6] * U[:, 6] + U[:, 7] * U[:, 7]))
    ref = P.criteria_grad(W, 2)
    assert np.array_equal(g[lf], ref[lf])
    assert np.all(g[~lf] == -1.0)
    iref, ico = sim.criteria_flags()
    eref, eco = P.criteria_flags(ref, lf, o.get("lp")[:, 0], kw["maxlevs"])
    assert np.array_equal(iref, eref) and np.array_equal(ico, eco)
    assert ico.any()   # the ambient region is uniform: its leaves are marked to coarsen


@pytest.mark.gpu
def test_set_tree_continues_a_run_bit_for_bit(gpu):
    """A run handed over mid-way (the oracle's quadtree, time state and the
    fields U, Bi, ff, gg after 20 steps, as a reference run would hand them)
    continues bit-identical to the oracle for 15 more steps, remeshing
    included."""
    kw = dict(ic="rotor", limiter="MC", flux="HLLD", cfl=0.4, maxlevs=4)
    o = P.Oracle(**kw).init()
    o.run(20)
    inf = o.info()
    sim = gpu.Simulation(**to_gpu_cfg(kw))   # created, not initialised
    sim.set_tree(o.get("lp"), o.get("icoord"), o.get("leafs"), inf["nbleafs"], inf["t"], inf["dt"],
                 inf["dt_next"], inf["count"])
    for f in ("U", "Bi", "ff", "gg"):
        sim.upload(f, o.get(f))
    o.run(35)
    sim.run(15)
    a, b = sim.state(), o.state()
    assert P.compare_states(a, b, 2)[0]
    assert np.array_equal(a["U"], b["U"]) and np.array_equal(a["Bi"], b["Bi"]) and a["t"] == b["t"]
    assert sim.info()["steps"] == 35
    with pytest.raises(gpu.AmrError):   # amr_set_tree takes the place of amr_init
        sim.set_tree(o.get("lp"), o.get("icoord"), o.get("leafs"), inf["nbleafs"], 0.0, 0.0, 0.0, 0)


@pytest.mark.gpu
def test_admesh_marked_matches_oracle(gpu):
    """amr_admesh_marked with arbitrary marks (the caller choosing the blocks
    to prolong and restrict) gives the oracle's tree and fields bit for bit
    after each remesh, and the run continues bit-identical."""
    kw = dict(ic="rotor", limiter="MC", flux="HLLD", cfl=0.4, maxlevs=4)
    sim = gpu.Simulation(**to_gpu_cfg(kw)).init()
    o = P.Oracle(**kw).init()
    rng = np.random.default_rng(3)
    changed = 0
    for k in range(4):
        sim.run(5)
        o.run(5 * (k + 1))
        n = o.info()["lastActive"]
        leaves = o.get("leafs").copy()
        iref, ico = rng.random(n) < 0.1, rng.random(n) < 0.7
        sim.admesh_marked(iref, ico)
        o.admesh_marked(iref, ico)
        a, b = sim.state(), o.state()
        changed += int(a["lastActive"] != n or not np.array_equal(a["leafs"][:n], leaves))
        assert P.compare_states(a, b, 2)[0], k
        assert np.array_equal(a["U"], b["U"]) and np.array_equal(a["Bi"], b["Bi"]), k
    assert changed >= 3
    sim.run(10)
    o.run(30)
    a, b = sim.state(), o.state()
    assert P.compare_states(a, b, 2)[0]
    assert np.array_equal(a["U"], b["U"]) and np.array_equal(a["Bi"], b["Bi"]) and a["t"] == b["t"]


@pytest.mark.gpu
def test_set_tree_refuses_a_broken_tree(gpu):
    """A handed tree whose neighbour link leaves the ID range is refused on
    the host (AMR_E_ARG) before any ID reaches the device; the instance then
    takes the intact tree."""
    kw = dict(ic="rotor", limiter="MC", flux="HLLD", cfl=0.4, maxlevs=4)
    o = P.Oracle(**kw).init()
    o.run(10)
    inf = o.info()
    lp = o.get("lp").copy()
    leaf = int(np.flatnonzero(o.get("leafs"))[-1])
    lp[leaf, 5] = inf["lastActive"] + 100
    sim = gpu.Simulation(**to_gpu_cfg(kw))
    with pytest.raises(gpu.AmrError) as e:
        sim.set_tree(lp, o.get("icoord"), o.get("leafs"), inf["nbleafs"], inf["t"], inf["dt"], inf["dt_next"],
                     inf["count"])
    assert e.value.code == -12
    sim.set_tree(o.get("lp"), o.get("icoord"), o.get("leafs"), inf["nbleafs"], inf["t"], inf["dt"],
                 inf["dt_next"], inf["count"])
    for f in ("U", "Bi", "ff", "gg"):
        sim.upload(f, o.get(f))
    o.run(12)
    sim.run(2)
    a, b = sim.state(), o.state()
    assert P.compare_states(a, b, 2)[0] and np.array_equal(a["U"], b["U"])


@pytest.mark.gpu
def test_remesh_off_then_admesh_is_a_step(gpu):
    """amr_set_remesh(0) + amr_step + amr_admesh equals amr_step bit for bit:
    the caller can act between the dt reduction and admesh, as main.cpp:240-246
    saves there."""
    kw = to_gpu_cfg(dict(ic="rotor", limiter="MC", flux="HLLD", cfl=0.4, maxlevs=4))
    a = gpu.Simulation(**kw).init()
    b = gpu.Simulation(**kw).init()
    b.set_remesh(False)
    for _ in range(25):
        a.step()
        b.step()
        b.admesh()
    sa, sb = a.state(), b.state()
    assert P.compare_states(sa, sb, 2)[0]
    assert np.array_equal(sa["U"], sb["U"]) and np.array_equal(sa["Bi"], sb["Bi"]) and sa["t"] == sb["t"]
