"""The C-ABI library: it loads without a GPU and exports every entry point
include/amr2d_mhd.h declares; configuration parsing and argument checks."""
import ctypes
import os
import re

import pytest

import amr2d_mhd_gb300 as amr

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared():
    src = open(os.path.join(REPO, "include", "amr2d_mhd.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(amr_[a-z0-9_]+)\s*\(", src)))


def test_exports_every_declared_symbol():
    L = amr.load()
    names = declared()
    assert len(names) >= 20
    for n in names:
        assert hasattr(L, n), n
    assert sorted(amr.EXPORTS) == names


def test_abi_version_and_status_strings():
    L = amr.load()
    assert L.amr_abi_version() == 1
    assert L.amr_status_string(-5) == b"zero or negative pressure"


def test_config_from_input_txt(tmp_path):
    p = tmp_path / "input.txt"
    p.write_text("16 16 8\n1.0 1.0 \n0.5\nrotor MC RUSA\n")  # the reference's shipped input.txt
    c = amr.make_config(input_txt=str(p))
    assert (c.nx, c.ny, c.nvar, c.cfl) == (16, 16, 8, 0.5)
    assert (c.ic, c.limiter, c.flux) == (b"rotor", b"MC", b"RUSA")
    assert c.maxlevs == 5 and c.nghosts == 2 and c.nroots_x == 2


def test_missing_input_txt(tmp_path):
    with pytest.raises(amr.AmrError) as e:
        amr.make_config(input_txt=str(tmp_path / "nope.txt"))
    assert e.value.code == -1


def test_create_rejects_bad_options_before_touching_the_gpu():
    L = amr.load()
    h = ctypes.c_void_p()
    for kw, code in [(dict(limiter="bogus"), -1), (dict(flux="ROE"), -11), (dict(flux="XYZ"), -1),
                     (dict(limiter="WENO5", nghosts=2), -1), (dict(nx=8, ny=8), -11), (dict(ic="nope"), -1),
                     (dict(ct_type=3), -1), (dict(ct_type=-1), -1), (dict(diffusion=2), -1)]:
        c = amr.make_config(**kw)
        assert L.amr_create(ctypes.byref(c), ctypes.byref(h)) == code, kw


def test_step_halves_need_an_initialised_handle():
    """amr_step_begin / amr_step_end on a NULL handle: argument error, no crash."""
    L = amr.load()
    assert L.amr_step_begin(None) == -12
    assert L.amr_step_end(None) == -12


def test_python_config_mirror_matches_the_c_struct():
    """The ctypes mirror of amr_config has the C layout's size (the library
    writes sizeof(amr_config) into struct_size) and the new fields land where
    the C code reads them (ct_type / diffusion validated by amr_create)."""
    c = amr.make_config(ct_type=2, diffusion=True)
    assert c.struct_size == ctypes.sizeof(amr.Config)
    assert (c.ct_type, c.diffusion, c.reserved[0], c.reserved[1]) == (2, 1, 0, 0)
    assert ctypes.sizeof(amr.Profile) == 8 * 12   # 12 eight-byte fields of amr_profile


def test_every_entry_point_rejects_a_null_handle():
    """Each call that takes a handle returns AMR_E_ARG for NULL (no crash, no
    device call); amr_destroy(NULL) is a no-op like free(NULL)."""
    L = amr.load()
    handle_first = {"amr_destroy", "amr_set_stream", "amr_last_error"} | {
        n for n in amr.EXPORTS
        if n not in ("amr_cfl_dt_static", "amr_riemann", "amr_config_default", "amr_config_from_input", "amr_config_blast",
                     "amr_config_kh", "amr_abi_version", "amr_status_string", "amr_create", "amr_create_batch")}
    assert "amr_criteria_flags" in handle_first and "amr_set_tree" in handle_first
    for n in sorted(handle_first):
        fn = getattr(L, n)
        args = [None] + [0 if t in (ctypes.c_int32, ctypes.c_int64, ctypes.c_size_t, ctypes.c_double) else None
                         for t in fn.argtypes[1:]]
        assert fn(*args) == (0 if n == "amr_destroy" else -12), n
    # the allocation-free CFL reduction checks its pointers before any launch
    assert L.amr_cfl_dt_static(None, 4, 2, None, 5 / 3, None, None) == -12
    # riemannS on arrays: pointers, solver and ROE's magnetic-field rejection
    # (riemannS.cpp:39-40) are checked before any device call
    w = (ctypes.c_double * 8)()
    assert L.amr_riemann(0, 0, 1, 1.4, None, w, w, None, 1) == -12
    assert L.amr_riemann(7, 0, 1, 1.4, w, w, w, None, 1) == -1
    assert L.amr_riemann(4, 0, 1, 1.4, w, w, w, None, 1) == -11
