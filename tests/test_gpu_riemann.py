"""riemannS on the GPU through the C ABI (amr_riemann) against the
reference's own answers: the known-answer cases of its riemannS / misc
objects (tests/golden/kat_riemann.npz, magnetic field on: RUSA, HLLE, HLLC,
HLLD, x and y faces) bit for bit, and those of its hydrodynamic build
(kat_riemann_hydro.npz, MAG_field = false), where ROE runs: the four MHD
solvers bit for bit, ROE to a few ulp (its pow(a, 2) against the correctly
rounded square)."""
import os

import numpy as np
import pytest

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
FLUXES = ["RUSA", "HLLE", "HLLC", "HLLD", "ROE"]


def _by_case(gpu, d, mag_field):
    out = np.zeros_like(d["out"])
    st = np.zeros(len(d["flux"]), np.int32)
    for fl in np.unique(d["flux"]):
        for dr in (0, 1):
            for g in np.unique(d["gamma"]):
                m = (d["flux"] == fl) & (d["dir"] == dr) & (d["gamma"] == g)
                if not m.any():
                    continue
                o, s = gpu.riemann(FLUXES[fl], d["wL"][m], d["wR"][m], g, dir_y=bool(dr), mag_field=mag_field)
                out[m], st[m] = o, s
    return out, st


@pytest.mark.gpu
def test_riemann_matches_reference_kat(gpu):
    d = np.load(os.path.join(GOLDEN, "kat_riemann.npz"))
    out, st = _by_case(gpu, d, True)
    assert np.array_equal(st, np.where(d["status"] != 0, -8, 0))
    ok = d["status"] == 0
    assert np.array_equal(out[ok].view(np.int64), d["out"][ok].view(np.int64))


@pytest.mark.gpu
def test_riemann_hydro_and_roe_match_reference_kat(gpu):
    d = np.load(os.path.join(GOLDEN, "kat_riemann_hydro.npz"))
    out, st = _by_case(gpu, d, False)
    assert not st.any()
    roe = d["flux"] == 4
    assert np.array_equal(out[~roe].view(np.int64), d["out"][~roe].view(np.int64))
    ref, got = d["out"][roe], out[roe]
    scale = np.abs(ref).max(axis=1, keepdims=True)
    assert np.all(np.abs(got - ref) <= 8 * np.finfo(np.float64).eps * scale)
    same = np.all(got.view(np.int64) == ref.view(np.int64), axis=1).mean()
    print("ROE cases bit-identical to the reference: %.3f" % same)
    assert same >= 0.9


@pytest.mark.gpu
def test_riemann_rejects_roe_with_magnetic_field(gpu):
    w = np.ones((1, 8))
    with pytest.raises(gpu.AmrError) as e:
        gpu.riemann("ROE", w, w, 1.4, mag_field=True)
    assert e.value.code == -11   # riemannS.cpp:39-40
