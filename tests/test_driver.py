"""The host program amr2d_mhd (the reference's main() on the library): what
it does before any device call, checked without a GPU."""
import os
import subprocess

import pytest

from amr2d_mhd_gb300 import build as B

INPUT = "16 16 8\n1.0 1.0 \n0.4\nBWx MC RUSA\n"


@pytest.fixture(scope="module")
def driver():
    B.build()   # builds the library and the driver when they are stale
    assert os.path.exists(B.DRIVER)
    return B.DRIVER


def run(driver, cwd, stdin="", *args):
    return subprocess.run([driver, *args], cwd=cwd, input=stdin, capture_output=True, text=True, timeout=60)


def test_usage(driver, tmp_path):
    r = run(driver, tmp_path, "", "--help")
    assert r.returncode == 0 and "usage: amr2d_mhd" in r.stdout


def test_bad_option(driver, tmp_path):
    r = run(driver, tmp_path, "", "--maxlevs", "x")
    assert r.returncode == 2 and "bad argument" in r.stderr


def test_missing_input_txt(driver, tmp_path):
    """main.cpp:66-70: no input.txt ends the program."""
    r = run(driver, tmp_path, "2\n0\n")
    assert r.returncode == 1 and "Unable to open the file..." in r.stdout


def test_plot_choice_and_wrong_selection(driver, tmp_path):
    """main.cpp:73-95: 1 = plot existing data (left to the reference's
    script), anything but 1 or 2 is an error; neither runs a simulation."""
    (tmp_path / "input.txt").write_text(INPUT)
    r = run(driver, tmp_path, "1\n")
    assert r.returncode == 0 and "call_plot.py" in r.stdout
    assert "Problems chosen: BWx" in r.stdout and "Limiter selected: MC" in r.stdout
    r = run(driver, tmp_path, "3\n")
    assert r.returncode == 1 and "Error as wrong selection!" in r.stdout
    assert not (tmp_path / "data").exists()


def test_driver_config_equals_the_python_one(tmp_path):
    """The configuration the driver builds from input.txt and its defaults
    (amr_config_default + amr_config_from_input, maxlevs 3, nghosts 2,
    ct_type 1, FP64) is byte for byte the one the Python API builds for the
    same problem, so their runs can be compared."""
    import ctypes

    import amr2d_mhd_gb300 as amr
    from parity_util import to_gpu_cfg
    (tmp_path / "input.txt").write_text(INPUT)
    L = amr.load()
    c = amr.Config()
    L.amr_config_default(ctypes.byref(c))
    assert L.amr_config_from_input(str(tmp_path / "input.txt").encode(), ctypes.byref(c)) == 0
    c.maxlevs, c.nghosts, c.ct_type, c.diffusion, c.precision = 3, 2, 1, 0, 0
    p = amr.make_config(**to_gpu_cfg(dict(ic="BWx", limiter="MC", flux="RUSA", cfl=0.4, maxlevs=3)))
    assert bytes(c) == bytes(p)
