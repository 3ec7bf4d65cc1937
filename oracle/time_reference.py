"""Test infrastructure, not product code: times the reference's own build
(serial, and the OpenMP build of its makefile, `make USE_OMP=1`, makefile:
15-19) beside the oracle's C restatement on the same host, same problem and
same thread counts: the rotor with gamma 5/3 (the bench's problem in the
reference's geometry, oracle/ref.mk ROTOR_G53=1), 5 levels, MUSCL-MC + HLLD,
CFL 0.4, the first `steps` steps from t = 0.  cell-updates/s = sum over steps
of the leaf cells before the step / wall seconds of the run.  Needs the
reference sources (AMR_REFERENCE_SRC).

    AMR_REFERENCE_SRC=<checkout> python oracle/time_reference.py [steps] [threads ...]
"""
from __future__ import annotations

import json
import os
import sys
import time

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))

from oracle import pyoracle, ref_runner  # noqa: E402


def time_reference(steps: int, threads: int, flavor: str):
    p, wd, log = ref_runner._start("rotor", "MC", "HLLD", 0.4, 5, steps, 2, 10 ** 9, flavor, 16, 16, None, threads,
                                   1, False, True, True)
    t0 = time.perf_counter()
    p.wait()
    sec = time.perf_counter() - t0
    log.close()
    tl = ref_runner.read_tlog(os.path.join(wd, "tlog.bin"))
    cells = sum(tl[k - 1][2] * 256 for k in range(1, len(tl)))
    for f in os.listdir(wd):
        os.remove(os.path.join(wd, f))
    os.rmdir(wd)
    return cells / sec, sec, len(tl) - 1


def time_port(steps: int, threads: int):
    o = pyoracle.Oracle(ic="rotor", limiter="MC", flux="HLLD", cfl=0.4, maxlevs=5, gamma=5.0 / 3.0,
                        nthreads=threads).init()
    cells = 0
    t0 = time.perf_counter()
    for _ in range(steps):
        cells += int(o.get("leafs").sum()) * 256
        o.step()
    return cells / (time.perf_counter() - t0)


def main():
    steps = int(sys.argv[1]) if len(sys.argv) > 1 else 200
    threads = [int(x) for x in sys.argv[2:]] or [1, os.cpu_count() or 1]
    pyoracle.build()
    out = {"problem": "rotor gamma 5/3, reference geometry, 5 levels, MUSCL-MC + HLLD, CFL 0.4, steps 1..%d" % steps,
           "host_cores": os.cpu_count(), "runs": []}
    for t in threads:
        flavor = "nofma" if t == 1 else "omp"
        ref, sec, n = time_reference(steps, t, flavor)
        port = time_port(steps, t)
        out["runs"].append({"threads": t, "reference_build": flavor, "reference_cell_updates_per_s": ref,
                            "port_cell_updates_per_s": port, "port_over_reference": port / ref,
                            "reference_seconds": sec, "reference_steps": n})
        print(json.dumps(out["runs"][-1]), flush=True)
    print(json.dumps(out))


if __name__ == "__main__":
    main()
