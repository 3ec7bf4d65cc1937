"""Generates the golden fixtures of tests/golden/ from the reference itself.

Needs the reference sources (spaceauk/AMR2D_MHD), named by the environment
variable AMR_REFERENCE_SRC: it builds the unmodified reference with oracle/ref.mk
(FLAVOR=nofma: the shipped makefile flags plus -ffp-contract=off, so that its
floating-point operations are not fused and every other implementation can
reproduce them exactly) and records

  run_<name>.npz    per-step fingerprints (tree and leaf-state SHA-256, t,
                    dt, leaf counts, per-variable sums) of a time loop;
  state_<name>.npz  one full state (lp, icoord, leafs, U, Bi) of a small run;
  kat_riemann.npz   riemannS() answers for seeded left / right states;
  kat_limiter.npz   slopelimiter() answers;
  kat_riemann_hydro.npz  riemannS() answers of the reference built with
                    MAG_field = false (defs.hpp:32), every solver including
                    ROE (riemannS.cpp:297-395), which only that build reaches;
  oracle_<name>.npz the same for a run the reference cannot make (the
                    bench's geometry: 16 x 16 cells of 1/32 on [0,1]^2),
                    made by the oracle (oracle/amr_oracle.c, itself pinned
                    to the reference by the fixtures above);
  long_<name>.npz   a run to its end time: t, dt and leaf counts of every
                    step, fingerprints every `every` steps and of the last
                    step (the bench's rotor, gamma 5/3, built with
                    ROTOR_G53=1).

Usage: python tests/golden/make_golden.py [name ...]
"""
import os
import struct
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, REPO)
sys.path.insert(0, HERE)

from golden_util import pack, record  # noqa: E402
from oracle import pyoracle, ref_runner  # noqa: E402

# name: (ic, limiter, flux, cfl, maxlevs, nghosts, steps)
RUNS = {
    "bw_L4_mc_rusa_full": ("BWx", "MC", "RUSA", 0.4, 4, 2, 100000),  # to t_end = 0.2
    "rotor_L5_mc_rusa_200": ("rotor", "MC", "RUSA", 0.4, 5, 2, 200),
    "rotor_L5_mc_hlld_100": ("rotor", "MC", "HLLD", 0.4, 5, 2, 100),
    "bw_L4_mc_hlle_60": ("BWx", "MC", "HLLE", 0.4, 4, 2, 60),
    "bw_L4_mc_hllc_60": ("BWx", "MC", "HLLC", 0.4, 4, 2, 60),
    "bwy_L3_minmod_hlld_40": ("BWy", "minmod", "HLLD", 0.4, 3, 2, 40),
    "bwx1_L3_vanleer_rusa_40": ("BWx1", "VanLeer", "RUSA", 0.4, 3, 2, 40),
    "sst_L3_superbee_hlle_40": ("SST", "Superbee", "HLLE", 0.4, 3, 2, 40),
    "ssty_L3_koren_rusa_40": ("SSTy", "Koren", "RUSA", 0.4, 3, 2, 40),
    "bwy1_L3_cada3rd_rusa_40": ("BWy1", "Cada3rd", "RUSA", 0.4, 3, 2, 40),
    "sst1_L3_1st_rusa_40": ("SST1", "1st", "RUSA", 0.4, 3, 2, 40),
    "bw_L3_nosl_rusa_20": ("BWx", "noSL", "RUSA", 0.2, 3, 2, 20),
    "bw_L3_weno3_rusa_40": ("BWx", "WENO3", "RUSA", 0.4, 3, 2, 40),
    "bw_L3_weno5_hlld_40": ("BWx", "WENO5", "HLLD", 0.4, 3, 4, 40),
    "rotor_L3_weno5_rusa_40": ("rotor", "WENO5", "RUSA", 0.4, 3, 4, 40),
    # compile-time options of the reference (defs.hpp:34-35), built with them
    "bw_L4_mc_rusa_ct2_100": ("BWx", "MC", "RUSA", 0.4, 4, 2, 100, dict(ct_type=2)),
    "rotor_L5_mc_hlld_ct2_60": ("rotor", "MC", "HLLD", 0.4, 5, 2, 60, dict(ct_type=2)),
    "bw_L4_mc_rusa_diff_100": ("BWx", "MC", "RUSA", 0.4, 4, 2, 100, dict(diffusion=True)),
    "rotor_L5_mc_hlld_ct2diff_60": ("rotor", "MC", "HLLD", 0.4, 5, 2, 60, dict(ct_type=2, diffusion=True)),
}
# name: (ic, limiter, flux, cfl, maxlevs, nghosts, every, build options)
LONG = {
    "rotor53_L5_mc_hlld": ("rotor", "MC", "HLLD", 0.4, 5, 2, 25, dict(rotor_g53=True)),
    "rotor53_L5_mc_rusa": ("rotor", "MC", "RUSA", 0.4, 5, 2, 25, dict(rotor_g53=True)),
}
STATES = {  # name: (ic, limiter, flux, cfl, maxlevs, nghosts, step)
    "bw_L2_mc_rusa_step10": ("BWx", "MC", "RUSA", 0.4, 2, 2, 10),
}


def make_run(name):
    ic, lim, fl, cfl, L, ng, steps = RUNS[name][:7]
    opts = RUNS[name][7] if len(RUNS[name]) > 7 else {}
    refs, wd = ref_runner.run(ic, lim, fl, cfl, L, steps, nghosts=ng, every=1, **opts)
    n = max(refs)
    recs = [record(refs[s], ng) for s in range(n + 1)]
    meta = dict(ic=ic, limiter=lim, flux=fl, cfl=cfl, maxlevs=L, nghosts=ng, steps=n, **opts)
    np.savez_compressed(os.path.join(HERE, "run_%s.npz" % name), meta=np.array(repr(meta)), **pack(recs))
    for f in os.listdir(wd):
        os.remove(os.path.join(wd, f))
    os.rmdir(wd)
    print(name, "steps", n, "t_end", recs[-1]["t"], "leaves", recs[-1]["nleaves"])


def make_long(name):
    ic, lim, fl, cfl, L, ng, every, opts = LONG[name]
    recs = {}

    def consume(step, st):
        recs[step] = record(st, ng)
        if step % (every * 40) == 0:
            print(name, "step", step, "t", st["t"], "leaves", recs[step]["nleaves"], flush=True)

    tlog, wd = ref_runner.run_stream(consume, ic, lim, fl, cfl, L, 10 ** 7, nghosts=ng, every=every, **opts)
    n = tlog[-1][0]
    assert [r[0] for r in tlog] == list(range(n + 1)), "time log has gaps"
    assert n in recs, "no dump of the last step"
    fp = sorted(recs)
    meta = dict(ic=ic, limiter=lim, flux=fl, cfl=cfl, maxlevs=L, nghosts=ng, steps=n, every=every, gamma=5.0 / 3.0,
                **opts)
    np.savez_compressed(os.path.join(HERE, "long_%s.npz" % name), meta=np.array(repr(meta)),
                        t=np.array([r[3] for r in tlog]), dt=np.array([r[4] for r in tlog]),
                        nleaves=np.array([r[2] for r in tlog], np.int32),
                        last_active=np.array([r[1] for r in tlog], np.int32),
                        fp_step=np.array(fp, np.int32), tree=np.array([recs[s]["tree"] for s in fp]),
                        leaf=np.array([recs[s]["leaf"] for s in fp]), sums=np.array([recs[s]["sums"] for s in fp]))
    for f in os.listdir(wd):
        os.remove(os.path.join(wd, f))
    os.rmdir(wd)
    print(name, "steps", n, "t_end", tlog[-1][3], "leaves", tlog[-1][2])


ORACLE_LONG = {  # name: oracle keywords, fingerprint every
    "rotor53_bench_L5_mc_hlld": (dict(ic="rotor", limiter="MC", flux="HLLD", cfl=0.4, maxlevs=5, nghosts=2,
                                      geom_ref=False, gamma=5.0 / 3.0), 250),
}


def make_oracle_long(name, nthreads=4):
    kw, every = ORACLE_LONG[name]
    o = pyoracle.Oracle(**kw, nthreads=nthreads).init()
    t, dt, nl, fps = [], [], [], {}
    s = 0
    while True:
        inf = o.info()
        t.append(inf["t"])
        dt.append(inf["dt"])
        nl.append(int(o.get("leafs").sum()))
        if s % every == 0 or o.done:
            fps[s] = record(o.state(), kw["nghosts"])
        if o.done:
            break
        o.step()
        s += 1
    fp = sorted(fps)
    meta = dict(kw, steps=s, every=every, made_by="oracle")
    np.savez_compressed(os.path.join(HERE, "oracle_%s.npz" % name), meta=np.array(repr(meta)), t=np.array(t),
                        dt=np.array(dt), nleaves=np.array(nl, np.int32), fp_step=np.array(fp, np.int32),
                        tree=np.array([fps[k]["tree"] for k in fp]), leaf=np.array([fps[k]["leaf"] for k in fp]),
                        sums=np.array([fps[k]["sums"] for k in fp]))
    print(name, "steps", s, "t_end", t[-1], "leaves", nl[-1])


def make_state(name):
    ic, lim, fl, cfl, L, ng, step = STATES[name]
    refs, wd = ref_runner.run(ic, lim, fl, cfl, L, step, nghosts=ng, every=step)
    st = refs[step]
    meta = dict(ic=ic, limiter=lim, flux=fl, cfl=cfl, maxlevs=L, nghosts=ng, step=step)
    np.savez_compressed(os.path.join(HERE, "state_%s.npz" % name), meta=np.array(repr(meta)), t=st["t"],
                        dt=st["dt"], lp=st["lp"], icoord=st["icoord"], leafs=st["leafs"], U=st["U"], Bi=st["Bi"])
    print(name, "blocks", st["lastActive"])


def _states(rng, n):
    w = np.empty((n, 8))
    w[:, 0] = rng.uniform(0.1, 10.0, n)
    w[:, 1:4] = rng.uniform(-2.0, 2.0, (n, 3))
    w[:, 4] = rng.uniform(0.05, 20.0, n)
    w[:, 5:8] = rng.uniform(-2.0, 2.0, (n, 3))
    return w


def make_kat_riemann():
    rng = np.random.default_rng(20240611)
    cases = []
    for fl in range(4):
        for d in range(2):
            n = 96
            wL, wR = _states(rng, n), _states(rng, n)
            kn = 5 if d == 0 else 6
            wR[: n // 2, kn] = wL[: n // 2, kn]        # continuous normal B, as under CT
            wR[n // 2: n // 2 + 8] = wL[n // 2: n // 2 + 8]  # identical states
            wL[n // 2 + 8: n // 2 + 12, 5:8] = 0.0     # no field
            wR[n // 2 + 8: n // 2 + 12, 5:8] = 0.0
            g = rng.choice([1.4, 5.0 / 3.0, 2.0], n)
            for q in range(n):
                cases.append((fl, d, g[q], wL[q], wR[q]))
    exe = os.path.join(os.path.dirname(ref_runner.build(5, 2, "nofma")), "kat.x")
    subprocess.check_call(["make", "-s", "-f", os.path.join(REPO, "oracle", "ref.mk"), "REF=" + ref_runner.ref_dir(),
                           "MAXLEVS=5", "NGHOSTS=2", "FLAVOR=nofma", "kat"], cwd=REPO, stderr=subprocess.DEVNULL)
    with tempfile.TemporaryDirectory() as td:
        fin, fout = os.path.join(td, "in"), os.path.join(td, "out")
        with open(fin, "wb") as f:
            for fl, d, g, a, b in cases:
                f.write(struct.pack("<iid", fl, d, g) + a.astype("<f8").tobytes() + b.astype("<f8").tobytes())
        subprocess.check_call([exe, "riemann", fin, fout])
        raw = open(fout, "rb").read()
    rec = np.dtype([("st", "<i4"), ("f", "<f8", 8)])
    out = np.frombuffer(raw, rec)
    np.savez_compressed(os.path.join(HERE, "kat_riemann.npz"),
                        flux=np.array([c[0] for c in cases], np.int32), dir=np.array([c[1] for c in cases], np.int32),
                        gamma=np.array([c[2] for c in cases]), wL=np.array([c[3] for c in cases]),
                        wR=np.array([c[4] for c in cases]), status=out["st"].copy(), out=out["f"].copy())
    print("kat_riemann", len(cases), "cases,", int(out["st"].sum()), "throw")


def make_kat_riemann_hydro():
    rng = np.random.default_rng(20261204)
    cases = []
    for fl in range(5):
        for d in range(2):
            n = 64
            wL, wR = _states(rng, n), _states(rng, n)
            wL[:, 5:8] = 0.0       # no field in the hydrodynamic configuration (meshblock.cpp:13)
            wR[:, 5:8] = 0.0
            wR[n // 2: n // 2 + 4] = wL[n // 2: n // 2 + 4]  # identical states
            g = rng.choice([1.4, 5.0 / 3.0, 2.0], n)
            for q in range(n):
                cases.append((fl, d, g[q], wL[q], wR[q]))
    subprocess.check_call(["make", "-s", "-f", os.path.join(REPO, "oracle", "ref.mk"), "REF=" + ref_runner.ref_dir(),
                           "MAXLEVS=5", "NGHOSTS=2", "FLAVOR=nofma", "MAGFIELD=false", "kat"], cwd=REPO,
                          stderr=subprocess.DEVNULL)
    exe = os.path.join(REPO, "oracle", "_ref", "L5_G2_nofma_HYDRO", "kat.x")
    with tempfile.TemporaryDirectory() as td:
        fin, fout = os.path.join(td, "in"), os.path.join(td, "out")
        with open(fin, "wb") as f:
            for fl, d, g, a, b in cases:
                f.write(struct.pack("<iid", fl, d, g) + a.astype("<f8").tobytes() + b.astype("<f8").tobytes())
        subprocess.check_call([exe, "riemann", fin, fout])
        raw = open(fout, "rb").read()
    rec = np.dtype([("st", "<i4"), ("f", "<f8", 8)])
    out = np.frombuffer(raw, rec)
    np.savez_compressed(os.path.join(HERE, "kat_riemann_hydro.npz"),
                        flux=np.array([c[0] for c in cases], np.int32), dir=np.array([c[1] for c in cases], np.int32),
                        gamma=np.array([c[2] for c in cases]), wL=np.array([c[3] for c in cases]),
                        wR=np.array([c[4] for c in cases]), status=out["st"].copy(), out=out["f"].copy())
    print("kat_riemann_hydro", len(cases), "cases,", int(out["st"].sum()), "throw")


def make_kat_limiter():
    r = np.concatenate([np.linspace(-3, 5, 161), [0.0, -0.0, 1.0, 2.0, 0.5, 1e-18, -1e-18, 1e6, -1e6, 3.0]])
    eta = [0.0, 0.5, 1.0 - 2e-15, 1.0 - 5e-16, 1.0, 1.0 + 5e-16, 1.0 + 2e-15, 3.0]
    cases = [(li, x, e if li == 7 else 0.0) for li in range(8) for x in r for e in (eta if li == 7 else [0.0])]
    exe = os.path.join(os.path.dirname(ref_runner.build(5, 2, "nofma")), "kat.x")
    with tempfile.TemporaryDirectory() as td:
        fin, fout = os.path.join(td, "in"), os.path.join(td, "out")
        with open(fin, "wb") as f:
            for li, x, e in cases:
                f.write(struct.pack("<idd", li, x, e))
        subprocess.check_call([exe, "limiter", fin, fout])
        phi = np.frombuffer(open(fout, "rb").read(), "<f8")
    np.savez_compressed(os.path.join(HERE, "kat_limiter.npz"), limiter=np.array([c[0] for c in cases], np.int32),
                        r=np.array([c[1] for c in cases]), eta=np.array([c[2] for c in cases]), phi=phi.copy())
    print("kat_limiter", len(cases), "cases")


if __name__ == "__main__":
    names = sys.argv[1:] or (["kat"] + list(STATES) + list(RUNS) + list(LONG) + list(ORACLE_LONG))
    pyoracle.build()
    if any(nm not in ORACLE_LONG for nm in names) and not ref_runner.available():
        sys.exit("reference sources not found (set AMR_REFERENCE_SRC)")
    for nm in names:
        if nm == "kat":
            make_kat_riemann()
            make_kat_limiter()
            make_kat_riemann_hydro()
        elif nm == "kat_hydro":
            make_kat_riemann_hydro()
        elif nm in STATES:
            make_state(nm)
        elif nm in LONG:
            make_long(nm)
        elif nm in ORACLE_LONG:
            make_oracle_long(nm)
        else:
            make_run(nm)
