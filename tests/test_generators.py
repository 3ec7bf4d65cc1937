"""Seeded problem generators of the C ABI (amr_config_blast, amr_config_kh)
against the restatement in tests/seeded.py, which is pinned by the C++
standard's known answer for std::mt19937_64."""
import ctypes

import pytest

import amr2d_mhd_gb300 as amr
from seeded import MT64, blast_params, kh_amplitudes


def test_mt19937_64_known_answer():
    # [rand.predef]: the 10000th output of a default-constructed
    # std::mt19937_64 (seed 5489) is 9981545732273789042
    g = MT64(5489)
    for _ in range(9999):
        g.raw()
    assert g.raw() == 9981545732273789042


@pytest.mark.parametrize("seed", [0, 1234, 2**40 + 7])
def test_blast_batch_draws(seed):
    levs = set()
    for i in range(64):
        c = amr.blast_config(seed, i)
        p, ml = blast_params(seed, i)
        assert list(c.ic_param[:6]) == p
        assert c.maxlevs == ml
        levs.add(ml)
        assert 0.05 <= p[0] < 0.15 and 5 <= p[1] < 50 and 3 <= ml <= 6
        assert c.ic == b"blast" and c.limiter == b"MC" and c.flux == b"HLLE"
        assert c.gamma == 1.4 and c.t_end == 0.1 and c.geometry == 1 and c.periodic == 0
    assert levs == {3, 4, 5, 6}


def test_kh_draws():
    c = amr.kh_config(42)
    assert list(c.ic_param[:16]) == pytest.approx(kh_amplitudes(42), rel=1e-15, abs=0)
    assert c.nroots_x == 16 and c.nroots_y == 16 and c.maxlevs == 1 and c.periodic == 1
    assert c.dt_fixed == 2e-4 and c.flux == b"RUSA" and c.limiter == b"MC"


def test_config_layout():
    c = amr.Config()
    amr.load().amr_config_default(ctypes.byref(c))
    assert c.struct_size == ctypes.sizeof(amr.Config)
    assert amr.Config.dt_fixed.offset % 8 == 0 and c.dt_fixed == 0.0
