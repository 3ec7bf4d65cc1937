"""Test infrastructure, not product code.

Builds (oracle/ref.mk) and runs the unmodified reference on an input.txt, and
returns its full-precision state dumps.  Needs the reference sources, found
through the environment variable AMR_REFERENCE_SRC (no default): without it
available() is False and nothing here runs.  The GPU machines use the
committed fixtures in tests/golden/ instead.
"""
from __future__ import annotations

import os
import struct
import subprocess
import tempfile
import time

from . import pyoracle

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)


def ref_dir() -> str:
    """The reference checkout named by AMR_REFERENCE_SRC ('' when unset)."""
    return os.environ.get("AMR_REFERENCE_SRC", "")


def available() -> bool:
    r = ref_dir()
    return bool(r) and os.path.isfile(os.path.join(r, "main.cpp"))


def build(maxlevs: int, nghosts: int = 2, flavor: str = "nofma", ct_type: int = 1, diffusion: bool = False,
          rotor_g53: bool = False) -> str:
    if not available():
        raise RuntimeError("reference sources not found: set AMR_REFERENCE_SRC")
    variant = ("_CT%d" % ct_type if ct_type != 1 else "") + ("_DIFF" if diffusion else "") + \
        ("_RG53" if rotor_g53 else "")
    out = os.path.join(HERE, "_ref", "L%d_G%d_%s%s" % (maxlevs, nghosts, flavor, variant), "main.x")
    subprocess.check_call(["make", "-s", "-j8", "-f", os.path.join(HERE, "ref.mk"),
                           "REF=" + ref_dir(), "MAXLEVS=%d" % maxlevs, "NGHOSTS=%d" % nghosts,
                           "FLAVOR=" + flavor, "CTTYPE=%d" % ct_type, "DIFFUSION=" + ("true" if diffusion else "false"),
                           "ROTOR_G53=%d" % (1 if rotor_g53 else 0)],
                          cwd=REPO, stderr=subprocess.DEVNULL)
    return out


def _start(ic, limiter, flux, cfl, maxlevs, steps, nghosts, every, flavor, nx, ny, workdir, threads, ct_type,
           diffusion, rotor_g53, tlog):
    exe = build(maxlevs, nghosts, flavor, ct_type, diffusion, rotor_g53)
    wd = workdir or tempfile.mkdtemp(prefix="amrref_")
    with open(os.path.join(wd, "input.txt"), "w") as f:
        f.write("%d %d 8\n1.0 1.0\n%r\n%s %s %s\n" % (nx, ny, cfl, ic, limiter, flux))
    env = dict(os.environ, AMR_REF_DUMP=os.path.join(wd, "d"), AMR_REF_EVERY=str(every),
               AMR_REF_STOP=str(steps), OMP_NUM_THREADS=str(threads))
    if tlog:
        env["AMR_REF_TLOG"] = os.path.join(wd, "tlog.bin")
    log = open(os.path.join(wd, "log.txt"), "w")
    p = subprocess.Popen([exe], stdin=subprocess.PIPE, cwd=wd, env=env, stdout=log, stderr=subprocess.STDOUT)
    p.stdin.write(b"2\n0\n")
    p.stdin.close()
    return p, wd, log


def run(ic: str, limiter: str, flux: str, cfl: float, maxlevs: int, steps: int,
        nghosts: int = 2, every: int = 1, flavor: str = "nofma", nx: int = 16, ny: int = 16,
        workdir: str | None = None, threads: int = 1, ct_type: int = 1, diffusion: bool = False,
        rotor_g53: bool = False):
    """Run the reference for `steps` steps; return {step: dump dict}."""
    p, wd, log = _start(ic, limiter, flux, cfl, maxlevs, steps, nghosts, every, flavor, nx, ny, workdir, threads,
                        ct_type, diffusion, rotor_g53, False)
    p.wait()
    log.close()
    res = {}
    for s in range(0, steps + 1, every):
        path = os.path.join(wd, "d_%d.bin" % s)
        if os.path.exists(path):
            res[s] = pyoracle.read_ref_dump(path)
    return res, wd


def read_tlog(path: str):
    """Records of AMR_REF_TLOG: list of (step, last_active, leaves, t, dt)."""
    raw = open(path, "rb").read()
    rec = struct.Struct("<iiiidd")
    out = []
    for o in range(0, len(raw) - rec.size + 1, rec.size):
        s, na, nl, _, t, dt = rec.unpack_from(raw, o)
        out.append((s, na, nl, t, dt))
    return out


def run_stream(consume, ic: str, limiter: str, flux: str, cfl: float, maxlevs: int, steps: int,
               nghosts: int = 2, every: int = 1, flavor: str = "nofma", ct_type: int = 1, diffusion: bool = False,
               rotor_g53: bool = False):
    """Run the reference with a dump every `every` steps, hand each dump to
    consume(step, dump) as soon as it is complete and delete it (a long run
    never holds more than two dumps on disk).  Returns the per-step time log
    (read_tlog) and the working directory."""
    p, wd, log = _start(ic, limiter, flux, cfl, maxlevs, steps, nghosts, every, flavor, 16, 16, None, 1, ct_type,
                        diffusion, rotor_g53, True)
    nxt = 0

    def take(s):
        path = os.path.join(wd, "d_%d.bin" % s)
        consume(s, pyoracle.read_ref_dump(path))
        os.remove(path)

    while True:
        done = p.poll() is not None
        # dump `nxt` is complete once a later one exists or the program ended
        while os.path.exists(os.path.join(wd, "d_%d.bin" % nxt)) and (
                done or os.path.exists(os.path.join(wd, "d_%d.bin" % (nxt + every)))):
            take(nxt)
            nxt += every
        if done:
            break
        time.sleep(0.5)
    log.close()
    # the last dump (AMR_REF_STOP or the end of the time loop) may be off the grid
    for f in sorted(os.listdir(wd)):
        if f.startswith("d_") and f.endswith(".bin"):
            take(int(f[2:-4]))
    return read_tlog(os.path.join(wd, "tlog.bin")), wd
