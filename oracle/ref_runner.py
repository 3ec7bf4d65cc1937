"""Test infrastructure, not product code.

Builds (oracle/ref.mk) and runs the unmodified reference on an input.txt, and
returns its full-precision state dumps.  Needs the reference sources, so it
only runs where they are mounted (REF below); the GPU machines use the
committed fixtures in tests/golden/ instead.
"""
from __future__ import annotations

import os
import subprocess
import tempfile

from . import pyoracle

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)
REF = os.environ.get("AMR_REFERENCE_SRC", "/root/reference")


def available() -> bool:
    return os.path.isfile(os.path.join(REF, "main.cpp"))


def build(maxlevs: int, nghosts: int = 2, flavor: str = "nofma", ct_type: int = 1, diffusion: bool = False) -> str:
    variant = ("_CT%d" % ct_type if ct_type != 1 else "") + ("_DIFF" if diffusion else "")
    out = os.path.join(HERE, "_ref", "L%d_G%d_%s%s" % (maxlevs, nghosts, flavor, variant), "main.x")
    subprocess.check_call(["make", "-s", "-j8", "-f", os.path.join(HERE, "ref.mk"),
                           "REF=" + REF, "MAXLEVS=%d" % maxlevs, "NGHOSTS=%d" % nghosts,
                           "FLAVOR=" + flavor, "CTTYPE=%d" % ct_type, "DIFFUSION=" + ("true" if diffusion else "false")],
                          cwd=REPO, stderr=subprocess.DEVNULL)
    return out


def run(ic: str, limiter: str, flux: str, cfl: float, maxlevs: int, steps: int,
        nghosts: int = 2, every: int = 1, flavor: str = "nofma", nx: int = 16, ny: int = 16,
        workdir: str | None = None, threads: int = 1, ct_type: int = 1, diffusion: bool = False):
    """Run the reference for `steps` steps; return {step: dump dict}."""
    exe = build(maxlevs, nghosts, flavor, ct_type, diffusion)
    wd = workdir or tempfile.mkdtemp(prefix="amrref_")
    with open(os.path.join(wd, "input.txt"), "w") as f:
        f.write("%d %d 8\n1.0 1.0\n%r\n%s %s %s\n" % (nx, ny, cfl, ic, limiter, flux))
    env = dict(os.environ, AMR_REF_DUMP=os.path.join(wd, "d"), AMR_REF_EVERY=str(every),
               AMR_REF_STOP=str(steps), OMP_NUM_THREADS=str(threads))
    with open(os.path.join(wd, "log.txt"), "w") as log:
        subprocess.run([exe], input=b"2\n0\n", cwd=wd, env=env, stdout=log,
                       stderr=subprocess.STDOUT, check=False)
    res = {}
    for s in range(0, steps + 1, every):
        p = os.path.join(wd, "d_%d.bin" % s)
        if os.path.exists(p):
            res[s] = pyoracle.read_ref_dump(p)
    return res, wd
