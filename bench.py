#!/usr/bin/env python
"""Throughput of the per-block finite-volume update on the MHD rotor.

Workload: the MHD rotor on [0,1]^2, gamma = 5/3, 4 root blocks of 16x16 cells,
5 refinement levels, MUSCL with the MC limiter, HLLD fluxes, constrained
transport, RK2, CFL 0.4, outflow boundaries.  The run is advanced (untimed) to
t = T0, where the AMR tree is developed; a bench step is then one full time
step (both RK stages with CT, all ghost fills, the CFL reduction and the
remesh).  `value` is leaf cell-updates per second of the plain FP64 path, with
the state resident in HBM; `e2e` is the same through the C ABI with the state
in host memory (uploaded before and downloaded after every step).  The FP32
bulk path, its density error against FP64 at t_end, and the CPU baseline
(the oracle's restatement of the reference, on the host cores) are reported
beside it.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

REPO = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, REPO)

T0 = 0.05                 # start of the timed region (simulated time)
WORKLOAD = dict(ic="rotor", limiter="MC", flux="HLLD", cfl=0.4, maxlevs=5, nghosts=2, nroots=(2, 2),
                periodic=False, geometry=1, gamma=5.0 / 3.0, t_end=0.0)
WORKLOAD_NAME = ("MHD rotor [0,1]^2 gamma=5/3, 4 roots of 16x16, 5 levels, MUSCL-MC + HLLD + CT, RK2, "
                 "CFL 0.4, outflow, time steps from t=%.2f" % T0)
METRIC = "cell-updates/s"
# compulsory DRAM bytes per interior leaf cell of one launch of the face-flux
# kernel (the dominant kernel): it reads the primitive state (8 words) and the
# normal face field (2 words) and writes the x and y fluxes (2 x 8 words)
FACE_BYTES_PER_CELL = {"fp64": 26 * 8, "fp32": 24 * 4 + 2 * 8}
STEP_BYTES_PER_CELL = {"fp64": 400, "fp32": 240}   # one full RK2 step incl. CT (compulsory)


def dist_env():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def reduce_over_ranks(ms, cells, device):
    """Replicas (one process per GPU, no exchange in the data path): the job's
    time is the slowest rank's, its work the sum over ranks.  Called on every
    rank of an initialised process group (NCCL on GPUs, gloo in the CPU tests)."""
    import torch
    import torch.distributed as dist
    t = torch.tensor([ms, float(cells)], dtype=torch.float64, device=device)
    mx = t.clone()
    dist.all_reduce(mx, op=dist.ReduceOp.MAX)
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return float(mx[0]), float(t[1])


L2_NOTE = ("L2 flushed before every timed step: 256 MB written on the launch stream outside the step's timing "
           "events (the state, ~10-20 MB, would otherwise stay in the 129 MB L2); batches: state above L2 (no flush)")


def bench_config(world):
    """The `config` object of both arms' lines (identical by construction)."""
    return {"workload": WORKLOAD_NAME, "parallelism": "replicas" if world > 1 else "1 GPU", "l2": L2_NOTE}


class L2Flush:
    """Writes 256 MB (more than the 129 MB L2) on `stream`, so that the next
    timed step finds none of its state in L2."""

    def __init__(self, stream):
        import torch
        self.torch = torch
        self.buf = torch.empty(64 * 2 ** 20, dtype=torch.float32, device="cuda")
        self.stream = stream
        self.v = 0.0

    def __call__(self):
        self.v += 1.0
        with self.torch.cuda.stream(self.stream):
            self.buf.fill_(self.v)


def timed_steps(step, n, stream, flush):
    """n calls of `step` (one time step each), the L2 flushed before each and
    each between its own CUDA events on the launch stream; summed ms."""
    import torch
    pairs = []
    for _ in range(n):
        flush()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        step()
        e1.record(stream)
        pairs.append((e0, e1))
    torch.cuda.synchronize()
    return sum(a.elapsed_time(b) for a, b in pairs)


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.idx = gpu_index
        self.rows = []
        self.proc = None

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.idx), "--query-gpu=" + self.FIELDS,
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.th = threading.Thread(target=self._read, daemon=True)
            self.th.start()
        except OSError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([c.strip() for c in line.split(",")])

    def stop(self):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
        out = {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": len(self.rows)}
        try:
            sm = [float(r[1]) for r in self.rows if len(r) >= 9]
            mx = [float(r[2]) for r in self.rows if len(r) >= 9]
            if sm:
                out["sm_mhz"] = statistics.median(sm)
                out["sm_max_mhz"] = max(mx)
            names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
            for q, nm in enumerate(names):
                if any(r[5 + q].lower() == "active" for r in self.rows if len(r) >= 9):
                    out["reasons"].append(nm)
        except (ValueError, IndexError):
            pass
        return out


def measured_peaks():
    p = os.path.join(REPO, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def profile_summary(name):
    """Per-cell DRAM bytes / FP64 flops of the stage kernel from the committed ncu summary."""
    p = os.path.join(REPO, "profiles", name)
    if not os.path.exists(p):
        return None
    with open(p) as f:
        return json.load(f)


def fp64_peak_tflops(torch):
    """Measured FP64 rate of this GPU: a cuBLAS DGEMM, best of 5."""
    n = 4096
    a = torch.randn(n, n, dtype=torch.float64, device="cuda")
    b = torch.randn(n, n, dtype=torch.float64, device="cuda")
    torch.mm(a, b)
    torch.cuda.synchronize()
    best = 1e9
    for _ in range(5):
        s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        s.record()
        torch.mm(a, b)
        e.record()
        torch.cuda.synchronize()
        best = min(best, s.elapsed_time(e))
    return 2.0 * n ** 3 / (best * 1e-3) / 1e12


def advance_to(sim, t_stop, chunk=50):
    while True:
        inf = sim.info()
        if inf["done"] or inf["t"] >= t_stop:
            return inf
        sim.run(chunk)


def run_ours(args):
    import torch

    import amr2d_mhd_gb300 as amr

    world, rank, local = dist_env()
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    stream = torch.cuda.current_stream()
    K, W = args.steps, args.warmup

    def barrier():
        if world > 1:
            torch.distributed.barrier()

    def make(precision):
        sim = amr.Simulation(precision=precision, **WORKLOAD)
        sim.set_stream(stream.cuda_stream)
        return sim.init()

    results = {}
    flush = L2Flush(stream)
    for prec in ("fp64", "fp32"):
        sim = make(prec)
        advance_to(sim, T0)
        tune = sim.autotune() if not args.no_tune else ""
        sim.run(W)
        clocks = ClockSampler(local) if prec == "fp64" else None
        if clocks:
            clocks.start()
        sim.profile(True)
        i0 = sim.info()
        barrier()
        torch.cuda.synchronize()
        ms = timed_steps(sim.step, K, stream, flush)
        torch.cuda.synchronize()
        barrier()
        i1 = sim.info()
        prof = sim.profile()
        clk = clocks.stop() if clocks else None
        cells = i1["cell_updates"] - i0["cell_updates"]
        if world > 1:
            ms, cells = reduce_over_ranks(ms, cells, "cuda")
        results[prec] = dict(ms=ms, cells=cells, prof=prof, clocks=clk, leaves=i1["n_leaves"],
                             steps=i1["steps"] - i0["steps"],
                             schedule=next((l[2:] for l in tune.splitlines() if l.startswith("*")), "default"))
        if prec == "fp64":
            # e2e through the C ABI with the state in host memory: page-locked
            # buffers (views of a growable pinned allocation), then the same
            # with ordinary pageable arrays
            pinned = {}

            def host_view(name, shape):
                n = int(np.prod(shape))
                if name not in pinned or pinned[name].size < n:
                    pinned[name] = torch.empty(2 * n, dtype=torch.float64, pin_memory=True).numpy()
                return pinned[name][:n].reshape(shape)

            def e2e_run(pin):
                U, B = sim.download("U"), sim.download("Bi")
                if pin:
                    pu, pb = host_view("U", U.shape), host_view("B", B.shape)
                    pu[...], pb[...] = U, B
                    U, B = pu, pb
                sim.profile(False)
                j0 = sim.info()
                sec = 0.0
                for _ in range(K):
                    flush()
                    torch.cuda.synchronize()
                    t0 = time.perf_counter()
                    sim.upload("U", U)
                    sim.upload("Bi", B)
                    sim.step()
                    na = sim.info()["last_active"]
                    U = sim.download("U", out=host_view("U", (na,) + U.shape[1:]) if pin else U)
                    B = sim.download("Bi", out=host_view("B", (na,) + B.shape[1:]) if pin else B)
                    sec += time.perf_counter() - t0
                j1 = sim.info()
                p2 = sim.profile()
                return dict(s=sec, cells=j1["cell_updates"] - j0["cell_updates"],
                            h2d=p2["h2d_bytes"] / K, d2h=p2["d2h_bytes"] / K)

            results["e2e"] = e2e_run(True)
            results["e2e_pageable"] = e2e_run(False)
        # accuracy at t_end (untimed): FP32 against FP64
        advance_to(sim, 1e9, chunk=500)
        inf = sim.info()
        results[prec]["t_end"] = inf["t"]
        results[prec]["rho"] = sim.uniform(0) if rank == 0 else None
        sim.close()
    if not args.no_batch:
        results["rotor_batch"] = run_rotor_batch(stream, args.batch_steps)
        results["batch"] = run_batch(stream, args.batch_steps, args.batch_advance)
        results["batch"]["fp32_two_handles_pipelined"] = run_batch_pipelined(args.batch_steps, args.batch_advance)
    if not args.no_adjoint:
        results["adjoint"] = run_adjoint(stream)
    if not args.no_ot:
        results["orszag_tang"] = run_orszag_tang(stream)
    return results, world, rank


ROTOR_BATCH = 64


def run_rotor_batch(stream, steps):
    """ROTOR_BATCH copies of the bench rotor in one handle (independent
    instances, each bit-identical to a single run), advanced untimed to T0,
    then `steps` timed batch steps, FP64 and FP32."""
    import torch

    import amr2d_mhd_gb300 as amr
    out = {}
    for prec in ("fp64", "fp32"):
        sim = amr.Simulation([amr.make_config(precision=prec, **WORKLOAD) for _ in range(ROTOR_BATCH)])
        sim.set_stream(stream.cuda_stream)
        sim.init()
        while sim.info(0)["t"] < T0:
            sim.run(50)
        tune = sim.autotune(2)
        sim.run(3)
        sim.profile(True)
        c0 = sum(sim.info(q)["cell_updates"] for q in range(ROTOR_BATCH))
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        sim.run(steps)
        e1.record(stream)
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1)
        c1 = sum(sim.info(q)["cell_updates"] for q in range(ROTOR_BATCH))
        p = sim.profile()
        out[prec] = dict(value=(c1 - c0) / (ms * 1e-3), ms_per_step=ms / steps,
                         schedule=next((l[2:] for l in tune.splitlines() if l.startswith("*")), "default"),
                         step_gpu_ms_per_step=p["step_gpu_ms"] / steps,
                         stage_kernel_ms_per_step=p["stage_ms"] / steps,
                         host_compile_ms_per_step=p["host_compile_ms"] / steps,
                         host_admesh_ms_per_step=p["host_admesh_ms"] / steps,
                         host_capture_ms_per_step=p["host_capture_ms"] / steps)
        sim.close()
    return out


BATCH_SEED = 2026
BATCH_N = 512


def run_batch_pipelined(steps, advance, prec="fp32"):
    """The blast batch as two handles of 256 instances, each on its own
    stream, stepped with amr_step_begin / amr_step_end interleaved so that
    one handle's host half of a step (remesh, ghost-program compile) runs
    while the other's step is on the GPU.  Timed on the host between device
    synchronisations (two streams)."""
    import torch

    import amr2d_mhd_gb300 as amr
    cfgs = [amr.blast_config(BATCH_SEED, i, prec) for i in range(BATCH_N)]
    sims = [amr.Simulation(cfgs[:BATCH_N // 2]).init(), amr.Simulation(cfgs[BATCH_N // 2:]).init()]
    a, b = sims

    def pipelined(n):
        a.step_begin()
        for k in range(n):
            b.step_begin()
            a.step_end()
            if k + 1 < n:
                a.step_begin()
            b.step_end()

    pipelined(advance)
    for s in sims:
        s.autotune(2)
    pipelined(3)

    def cells():
        return sum(s.info(q)["cell_updates"] for s in sims for q in range(BATCH_N // 2))

    c0 = cells()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    pipelined(steps)
    torch.cuda.synchronize()
    sec = time.perf_counter() - t0
    c1 = cells()
    for s in sims:
        s.close()
    return dict(value=(c1 - c0) / sec, ms_per_step=sec * 1e3 / steps,
                workload="the same 512 instances as two handles of 256, host and device halves of their "
                         "steps interleaved (amr_step_begin / amr_step_end), %d timed steps" % steps)


def run_batch(stream, steps, advance):
    """The seeded blast batch (512 instances, maxlevs 3..6, MUSCL-MC + HLLE + CT,
    CFL 0.2): `advance` untimed batch steps, then `steps` timed ones, each one
    time step of every unfinished instance, in FP64 and FP32.  Accuracy: four
    instances (at most 4 levels) run to t = 0.1 in both precisions."""
    import torch

    import amr2d_mhd_gb300 as amr
    out = {}
    for prec in ("fp64", "fp32"):
        sim = amr.Simulation([amr.blast_config(BATCH_SEED, i, prec) for i in range(BATCH_N)])
        sim.set_stream(stream.cuda_stream)
        sim.init()
        sim.run(advance)
        tune = sim.autotune(2)
        sim.profile(True)
        c0 = sum(sim.info(q)["cell_updates"] for q in range(BATCH_N))
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        sim.run(steps)
        e1.record(stream)
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1)
        c1 = sum(sim.info(q)["cell_updates"] for q in range(BATCH_N))
        p = sim.profile()
        out[prec] = dict(value=(c1 - c0) / (ms * 1e-3), ms_per_step=ms / steps,
                         leaves=sum(sim.info(q)["n_leaves"] for q in range(BATCH_N)),
                         host_ms_per_step=(p["host_compile_ms"] + p["host_admesh_ms"]) / steps,
                         host_compile_ms_per_step=p["host_compile_ms"] / steps,
                         host_admesh_ms_per_step=p["host_admesh_ms"] / steps,
                         step_gpu_ms_per_step=p["step_gpu_ms"] / steps,
                         stage_kernel_ms_per_step=p["stage_ms"] / steps,
                         gpu_launches=int(p["launches"]),
                         launches_per_step=round(int(p["launches"]) / max(int(p["steps"]), 1), 2),
                         schedule=next((l[2:] for l in tune.splitlines() if l.startswith("*")), "default"))
        sim.close()
    l1 = []
    sims = {}
    for prec in ("fp64", "fp32"):
        cf = []
        for i in range(4):
            c = amr.blast_config(BATCH_SEED, i, prec)
            c.maxlevs = min(c.maxlevs, 4)
            cf.append(c)
        sims[prec] = amr.Simulation(cf).init()
        sims[prec].run()
    for i in range(4):
        a, b = sims["fp32"].uniform(0, instance=i), sims["fp64"].uniform(0, instance=i)
        l1.append(float(np.abs(a - b).sum() / np.abs(b).sum()))
    for v in sims.values():
        v.close()
    out["l1_rel_density_fp32_vs_fp64_max"] = max(l1)
    return out


OT_RUNS = ((3, "WENO5", 0.003), (4, "MC", 0.0015))


def ot_runs_at(levels, dt_scale=1.0):
    """MUSCL-MC + HLLD runs at the given levels, dt halved per level from the
    4-level run's 0.0015 (the finest cells set the stable step), times
    dt_scale."""
    return [(ml, "MC", dt_scale * 0.0015 * 2.0 ** (4 - ml)) for ml in levels]


class OTFailed(RuntimeError):
    """An Orszag-Tang run stopped by the library (e.g. negative pressure), with its time."""


def run_orszag_tang(stream, runs=OT_RUNS, t_end=None):
    """Orszag-Tang to t = pi (or t_end) in FP64 and in FP32 on a common fixed
    time grid; relative L1 difference of every conserved variable on the
    finest uniform grid, and the throughput of both paths."""
    import torch

    import amr2d_mhd_gb300 as amr
    out = []
    flush = L2Flush(stream)
    for ml, lim, dt in runs:
        res, rate = {}, {}
        for prec in ("fp64", "fp32"):
            cfg = amr.ot_config(ml, prec, limiter=lim, dt_fixed=dt)
            if t_end:
                cfg.t_end = t_end
            sim = amr.Simulation(cfg)
            sim.set_stream(stream.cuda_stream)
            sim.init()
            torch.cuda.synchronize()
            ms = 0.0
            try:
                while not sim.info()["done"]:   # steps past the end are no-ops
                    ms += timed_steps(sim.step, 50, stream, flush)
            except amr.AmrError as e:
                raise OTFailed("%s: %s at t in (%.6g, %.6g]" % (prec, e, sim.info()["t"], sim.info()["t"] + 50 * dt))
            inf = sim.info()
            rate[prec] = inf["cell_updates"] / (ms * 1e-3)
            res[prec] = [sim.uniform(k) for k in range(8)]
            steps = inf["steps"]
            sim.close()
        names = ["rho", "mx", "my", "mz", "E", "Bx", "By", "Bz"]
        l1 = {names[k]: float(np.abs(res["fp32"][k] - res["fp64"][k]).sum() / np.abs(res["fp64"][k]).sum())
              for k in range(8) if np.abs(res["fp64"][k]).sum() > 0}
        out.append(dict(maxlevs=ml, limiter=lim, flux="HLLD", dt=dt, steps=steps, t_end=t_end or "pi",
                        effective_grid=64 * 2 ** (ml - 1), fp64_cell_updates_per_s=rate["fp64"],
                        fp32_cell_updates_per_s=rate["fp32"], rel_l1_fp32_vs_fp64=l1))
    return out


KH_SEED = 42


def kh_u0(a, icoord, gamma=5.0 / 3.0, n=256, ng=2, nb=16):
    """Block-layout conserved state of the KH problem with amplitudes a (the
    IC of amr_config_kh, evaluated here so it can be perturbed)."""
    N = nb + 2 * ng
    idx = np.arange(N) - ng
    U = np.zeros((len(icoord), 8, N, N))
    k = np.arange(1, 17)
    for b, (x0, y0) in enumerate(icoord):
        x = (((x0 + idx) % n) + 0.5) / n
        y = (((y0 + idx) % n) + 0.5) / n
        Y, X = np.meshgrid(y, x, indexing="ij")   # [j][i]
        inside = np.abs(Y - 0.5) <= 0.25
        rho = np.where(inside, 2.0, 1.0)
        u = np.where(inside, 0.5, -0.5)
        env = np.exp(-(Y - 0.25) ** 2 / 0.01) + np.exp(-(Y - 0.75) ** 2 / 0.01)
        v = np.tensordot(a, np.sin(2.0 * np.pi * k[:, None, None] * X[None]), axes=1) * env
        bx = 0.1 / np.sqrt(4.0 * np.pi)
        U[b, 0], U[b, 1], U[b, 2] = rho, rho * u, rho * v
        U[b, 4] = 2.5 / (gamma - 1) + 0.5 * rho * (u * u + v * v) + 0.5 * bx * bx
        U[b, 5] = bx
    return U


def run_adjoint(stream, steps=200):
    """Gradient of the KH loss (total density in [0.4,0.6]^2 after `steps`
    steps of dt 2e-4 on the frozen 256^2 periodic mesh) w.r.t. the 16
    perturbation amplitudes: adjoint cost against a forward step, and the
    gradient against central differences (h = 1e-7); the same for the
    kinetic energy of the transverse motion (h = 1e-6 and 1e-7)."""
    import torch

    import amr2d_mhd_gb300 as amr
    c = amr.kh_config(KH_SEED)
    c.t_end = 1e9
    a0 = np.array(c.ic_param[:16])
    sim = amr.Simulation(c)
    sim.set_stream(stream.cuda_stream)
    sim.init()
    ic = sim.tree()[1]
    B0 = sim.download("Bi")
    ng, nb = 2, 16
    mask = np.zeros((len(ic), 20, 20))
    cc = (np.arange(20) - ng + 0.5)
    for b, (x0, y0) in enumerate(ic):
        x = (x0 + cc) / 256.0
        y = (y0 + cc) / 256.0
        inx, iny = (x >= 0.4) & (x <= 0.6), (y >= 0.4) & (y <= 0.6)
        m = np.outer(iny, inx).astype(float) / 256.0 ** 2
        m[:ng, :] = 0; m[-ng:, :] = 0; m[:, :ng] = 0; m[:, -ng:] = 0
        mask[b] = m

    flush = L2Flush(stream)

    def forward(a, record=False, timed=False):
        sim.upload("U", kh_u0(a, ic))
        sim.upload("Bi", B0)
        sim.adjoint_enable(record)
        torch.cuda.synchronize()
        if timed:
            ms = timed_steps(sim.step, steps, stream, flush)
        else:
            sim.run(steps)
            ms = 0.0
        U = sim.download("U")
        return float((U[:, 0] * mask).sum()), ms

    forward(a0)                                   # warm-up (graph capture)
    _, fwd_ms = forward(a0, timed=True)
    L, rec_ms = forward(a0, record=True, timed=True)
    lam = np.zeros((len(ic), 8, 20, 20))
    lam[:, 0] = mask
    sim.adjoint_seed("U", lam)
    torch.cuda.synchronize()
    adj_ms = timed_steps(sim.adjoint_step, steps, stream, flush)
    gU = sim.adjoint_read("U")

    def grad_a(gU):
        # chain rule through the IC: U2 = rho v, U4 = ... + rho v^2 / 2
        k = np.arange(1, 17)
        out = np.zeros(16)
        for b, (x0, y0) in enumerate(ic):
            x = (((x0 + np.arange(20) - ng) % 256) + 0.5) / 256
            y = (((y0 + np.arange(20) - ng) % 256) + 0.5) / 256
            Y, X = np.meshgrid(y, x, indexing="ij")
            rho = np.where(np.abs(Y - 0.5) <= 0.25, 2.0, 1.0)
            env = np.exp(-(Y - 0.25) ** 2 / 0.01) + np.exp(-(Y - 0.75) ** 2 / 0.01)
            basis = np.sin(2.0 * np.pi * k[:, None, None] * X[None]) * env    # dv/da_k
            v = np.tensordot(a0, basis, axes=1)
            out += (basis * (gU[b, 2] * rho + gU[b, 4] * rho * v)[None]).sum(axis=(1, 2))
        return out

    def fd_of(loss_of, h):
        fd = np.zeros(16)
        for q in range(16):
            e = np.zeros(16)
            e[q] = h
            fd[q] = (loss_of(a0 + e) - loss_of(a0 - e)) / (2 * h)
        return fd

    g = grad_a(gU)
    fd = fd_of(lambda a: forward(a)[0], 1e-7)
    # second loss: kinetic energy of the transverse motion, sum of m_y^2 / rho
    # dA over the interior; it scales with the perturbation, so central
    # differences resolve its gradient far below the kink error of the first
    inner = np.zeros((len(ic), 20, 20))
    inner[:, ng:-ng, ng:-ng] = 1.0 / 256.0 ** 2

    def ke_loss(a, record=False):
        forward(a, record)
        U = sim.download("U")
        return float((U[:, 2] ** 2 / U[:, 0] * inner).sum()), U

    _, U = ke_loss(a0, record=True)
    lam = np.zeros((len(ic), 8, 20, 20))
    lam[:, 2] = 2 * U[:, 2] / U[:, 0] * inner
    lam[:, 0] = -(U[:, 2] / U[:, 0]) ** 2 * inner
    sim.adjoint_seed("U", lam)
    for _ in range(steps):
        sim.adjoint_step()
    g_ke = grad_a(sim.adjoint_read("U"))
    fd_ke = {h: fd_of(lambda a: ke_loss(a)[0], h) for h in (1e-6, 1e-7)}
    sim.close()
    return dict(forward_ms_per_step=fwd_ms / steps, recording_ms_per_step=rec_ms / steps,
                adjoint_ms_per_step=adj_ms / steps, cost_ratio=adj_ms / fwd_ms, loss=L,
                grad_max_abs=float(np.abs(g).max()),
                fd_max_rel_diff=float(np.abs(g - fd).max() / np.abs(fd).max()),
                ke_loss={"loss": "sum of m_y^2 / rho dA over the domain after the same 200 steps",
                         "grad_max_abs": float(np.abs(g_ke).max()),
                         "fd_max_rel_diff_h1e-6": float(np.abs(g_ke - fd_ke[1e-6]).max() / np.abs(fd_ke[1e-6]).max()),
                         "fd_max_rel_diff_h1e-7": float(np.abs(g_ke - fd_ke[1e-7]).max() / np.abs(fd_ke[1e-7]).max())})


def cpu_baseline(steps, threads):
    """The oracle (the CPU restatement of the reference) on the host cores:
    the same rotor advanced to T0 (untimed), then `steps` timed steps."""
    from oracle import pyoracle as P
    o = P.Oracle(ic="rotor", limiter="MC", flux="HLLD", cfl=0.4, maxlevs=5, geom_ref=False, gamma=5.0 / 3.0,
                 nthreads=threads).init()
    while o.info()["t"] < T0:
        o.step()
    cells = 0
    t0 = time.perf_counter()
    for _ in range(steps):
        nl = int(o.get("leafs").sum())
        o.step()
        cells += nl * 256
    dt = time.perf_counter() - t0
    return cells / dt, dict(steps=steps, t0=T0, leaves=int(o.get("leafs").sum()), seconds=dt)


def run_reference(args):
    world, rank, _ = dist_env()
    if rank != 0:
        return 0
    threads = os.cpu_count() or 1
    from oracle import pyoracle as P
    o = P.Oracle(ic="rotor", limiter="MC", flux="HLLD", cfl=0.4, maxlevs=5, geom_ref=False, gamma=5.0 / 3.0,
                 nthreads=threads).init()
    while o.info()["t"] < T0:
        o.step()
    for _ in range(args.warmup):
        o.step()
    cells = 0
    t0 = time.perf_counter()
    for _ in range(args.steps):
        nl = int(o.get("leafs").sum())
        o.step()
        cells += nl * 256
    sec = time.perf_counter() - t0
    v = cells / sec
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": "cell-updates/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": sec / args.steps * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (rotor initial condition)",
            "config": bench_config(world),
            "cpu_baseline": {"value": v, "unit": "cell-updates/s", "cores": threads, "kind": "port",
                             "sample": "%d rotor time steps from t=%.2f on %d threads (oracle/amr_oracle.c, "
                                       "the C restatement of the reference)" % (args.steps, T0, threads)},
            "e2e": {"value": v, "unit": "cell-updates/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=300)
    ap.add_argument("--warmup", type=int, default=20)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--cpu-steps", type=int, default=40, help="steps of the CPU baseline sample")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-batch", action="store_true", help="skip the blast-batch measurement")
    ap.add_argument("--no-adjoint", action="store_true", help="skip the adjoint measurement")
    ap.add_argument("--no-tune", action="store_true", help="keep the default launch schedule")
    ap.add_argument("--no-ot", action="store_true", help="skip the Orszag-Tang precision comparison")
    ap.add_argument("--batch-steps", type=int, default=20)
    ap.add_argument("--batch-advance", type=int, default=120)
    ap.add_argument("--ncu-case", type=int, default=0,
                    help="profiling case: the rotor from its initial condition for this many steps, then exit")
    ap.add_argument("--ncu-t0", type=float, default=0.0,
                    help="with --ncu-case / --ncu-rotor-batch: first advance to this time (untimed), then run the steps")
    ap.add_argument("--precision", default="fp64", choices=["fp64", "fp32"], help="precision of --ncu-case")
    ap.add_argument("--ncu-tune", action="store_true",
                    help="with --ncu-case: run the autotuner before the profiled steps (the bench's schedule)")
    ap.add_argument("--ncu-rotor-batch", type=int, default=0,
                    help="profiling case: the %d-rotor batch, fused stage kernel, this many steps, then exit"
                         % ROTOR_BATCH)
    ap.add_argument("--ot-levels", default="",
                    help="only the Orszag-Tang FP32-vs-FP64 comparison, MUSCL-MC + HLLD at these levels "
                         "(comma-separated, e.g. 5,6), one JSON line")
    ap.add_argument("--ot-dt-scale", type=float, default=1.0, help="with --ot-levels: scale of the fixed dt")
    ap.add_argument("--ot-t-end", type=float, default=0.0, help="with --ot-levels: end time (default pi)")
    ap.add_argument("--adjoint-case", type=int, default=0,
                    help="profiling case: this many recorded and reversed steps of the KH adjoint, then exit")
    args = ap.parse_args()
    if args.ot_levels:
        import torch
        levels = [int(x) for x in args.ot_levels.split(",")]
        runs = []
        for ml in levels:   # one level at a time: a level that fails leaves the others' results
            try:
                runs += run_orszag_tang(torch.cuda.current_stream(), ot_runs_at([ml], args.ot_dt_scale),
                                        args.ot_t_end or None)
            except Exception as e:  # noqa: BLE001 - reported in the line
                runs.append({"maxlevs": ml, "limiter": "MC", "flux": "HLLD",
                             "dt": ot_runs_at([ml], args.ot_dt_scale)[0][2], "error": str(e)})
        print(json.dumps({"orszag_tang": runs, "workload": "Orszag-Tang on [0,2pi]^2, periodic, 4x4 roots of "
                          "16x16, gamma 5/3, MUSCL-MC + HLLD + CT, RK2, to t=pi on a fixed dt shared by both "
                          "precisions; FP32 bulk vs FP64, relative L1 per conserved variable on the finest "
                          "uniform grid"}))
        return 0
    if args.adjoint_case:
        import amr2d_mhd_gb300 as amr
        sim = amr.Simulation(amr.kh_config(5)).init()
        sim.run(4)
        sim.adjoint_enable(True)
        sim.run(args.adjoint_case)
        U = sim.download("U")
        lam = np.zeros_like(U)
        lam[:, 0] = 1.0
        sim.adjoint_seed("U", lam)
        for _ in range(args.adjoint_case):
            sim.adjoint_step()
        print(json.dumps(sim.info()))
        return 0
    if args.ncu_rotor_batch:
        import amr2d_mhd_gb300 as amr
        os.environ["AMR2D_STAGE_KERNEL"] = "fused"
        sim = amr.Simulation([amr.make_config(precision=args.precision, **WORKLOAD) for _ in range(ROTOR_BATCH)])
        sim.init()
        sim.profile(True)
        if args.ncu_t0 > 0:
            while sim.info(0)["t"] < args.ncu_t0:
                sim.run(50)
        before = sim.profile()["launches"]
        sim.run(args.ncu_rotor_batch)
        print(json.dumps(dict(sim.info(), launches_before=before, launches=sim.profile()["launches"] - before)))
        return 0
    if args.ncu_case:
        import amr2d_mhd_gb300 as amr
        sim = amr.Simulation(precision=args.precision, **WORKLOAD).init()
        sim.profile(True)
        if args.ncu_t0 > 0:
            advance_to(sim, args.ncu_t0)
        sched = sim.autotune() if args.ncu_tune else ""
        before = sim.profile()["launches"]
        sim.run(args.ncu_case)
        print(json.dumps(dict(sim.info(), launches_before=before, launches=sim.profile()["launches"] - before,
                              schedule=next((l[2:] for l in sched.splitlines() if l.startswith("*")), "default"))))
        return 0
    args.warmup = max(args.warmup, 3)
    if args.impl == "reference":
        return run_reference(args)

    import torch
    res, world, rank = run_ours(args)
    if rank != 0:
        return 0
    r64, r32, e2e = res["fp64"], res["fp32"], res["e2e"]
    value = r64["cells"] / (r64["ms"] * 1e-3)
    value32 = r32["cells"] / (r32["ms"] * 1e-3)
    # density error FP32 vs FP64 at t_end on the finest uniform grid
    a, b = r32["rho"], r64["rho"]
    l1 = float(np.abs(a - b).sum() / np.abs(b).sum())
    # roofline of the dominant kernel, the FP64 face-flux kernel: bound by
    # the FP64 pipe (GB300 issues 2 FP64 FMA per SM per clock), so the
    # primary roofline is its FP64 flop rate against a measured DGEMM; the
    # HBM view (algorithmic bytes against the measured copy bandwidth) is
    # reported beside it
    prof = r64["prof"]
    stage_ms_avg = max(prof["stage_ms"] / max(prof["stage_launches"], 1), 1e-9)
    cells_per_launch = prof["stage_cells"] / max(prof["stage_launches"], 1)
    alg_bytes = cells_per_launch * FACE_BYTES_PER_CELL["fp64"]
    achieved = alg_bytes / (stage_ms_avg * 1e-3) / 1e9
    peak, peak_kind = measured_peaks()
    ps = profile_summary("faces_fp64_rotor_hlld.json")
    traffic = ps["dram_bytes_per_cell"] * cells_per_launch if ps else None
    fp64 = {}
    try:
        fp64["peak_tflops_dgemm"] = fp64_peak_tflops(torch)
        if ps and "dp_flops_per_cell" in ps:
            fp64["flops_per_launch"] = ps["dp_flops_per_cell"] * cells_per_launch
            fp64["achieved_tflops"] = fp64["flops_per_launch"] / (stage_ms_avg * 1e-3) / 1e12
            fp64["frac"] = fp64["achieved_tflops"] / fp64["peak_tflops_dgemm"]
        if ps and "fp64_pipe_inst_per_face" in ps and r64["clocks"]:
            # issue slots of the FP64 pipe: 2 thread-instructions per SM per clock
            sms = torch.cuda.get_device_properties(0).multi_processor_count
            slots = 2.0 * sms * r64["clocks"]["sm_mhz"] * 1e6 * stage_ms_avg * 1e-3
            faces = cells_per_launch / 256.0 * 578.0      # 2 x 17 x 17 faces per 16 x 16 block
            fp64["pipe_busy_frac"] = ps["fp64_pipe_inst_per_face"] * faces / slots
            fp64["arith_issue_frac"] = ps["fp64_arith_inst_per_face"] * faces / slots
            fp64["issue_note"] = ("FP64-pipe instructions per face from ncu (profiles/faces_fp64_rotor_hlld.md) x faces "
                                  "per launch / (2 x SMs x SM clock x launch time); DGEMM-relative frac counts an FMA as "
                                  "2 flops per issue slot, this kernel issues mostly DADD / DMUL")
    except Exception as ex:  # noqa: BLE001
        fp64["error"] = str(ex)
    sched = r64["schedule"]
    face_kernel = ("k_stage<2,MUSCL,HLLD,double>" if sched.startswith("fused") else
                   "k_faces_dyn<2,MUSCL,HLLD,double>" if " dynamic" in sched else
                   "k_faces_persist<2,MUSCL,HLLD,double>" if " persistent" in sched else "k_faces<2,MUSCL,HLLD,double>")
    hbm_view = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                "peak_source": peak_kind, "traffic": traffic, "bytes_per_launch": alg_bytes}
    if "frac" in fp64:
        roofline = {"bound": "fp64", "achieved": fp64["achieved_tflops"], "peak": fp64["peak_tflops_dgemm"],
                    "unit": "TFLOP/s", "frac": fp64["frac"], "peak_source": "measured (cuBLAS DGEMM 4096^3, this run)",
                    "traffic": traffic, "kernel": face_kernel, "launch_ms": stage_ms_avg,
                    "flops_per_launch": fp64["flops_per_launch"],
                    "note": "FP64 flops per cell from ncu (DADD + DMUL + 2 DFMA, profiles/faces_fp64_rotor_hlld.md) x "
                            "cells per launch / CUDA-event launch time; the kernel's HBM fraction is in `hbm`",
                    "hbm": hbm_view}
    else:
        roofline = dict(hbm_view, kernel=face_kernel, launch_ms=stage_ms_avg)
    cpu = None
    if not args.no_cpu and world == 1:
        threads = os.cpu_count() or 1
        v, info = cpu_baseline(args.cpu_steps, threads)
        cpu = {"value": v, "unit": "cell-updates/s", "cores": threads, "kind": "port",
               "sample": "%d rotor time steps from t=%.2f (%d leaves), oracle/amr_oracle.c on %d threads"
                         % (info["steps"], T0, info["leaves"], threads)}
    clk = r64["clocks"] or {}
    line = {
        "metric": METRIC, "value": value, "unit": "cell-updates/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": r64["ms"] / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (rotor initial condition)",
        "config": bench_config(world),
        "leaves": r64["leaves"],
        "e2e": {"value": e2e["cells"] / e2e["s"], "unit": "cell-updates/s",
                "h2d_bytes_per_step": int(e2e["h2d"]), "d2h_bytes_per_step": int(e2e["d2h"]),
                "host_memory": "page-locked (pinned) arrays",
                "pageable_value": res["e2e_pageable"]["cells"] / res["e2e_pageable"]["s"]},
        "roofline": roofline,
        "fp64_pipe": fp64,
        "schedule": r64["schedule"],
        "host_compile_ms_per_step": prof["host_compile_ms"] / args.steps,
        "host_capture_ms_per_step": prof["host_capture_ms"] / args.steps,
        "step_gpu_ms_per_step": prof["step_gpu_ms"] / args.steps,
        "fp32": {"value": value32, "speedup_vs_fp64": value32 / value, "l1_rel_density_vs_fp64_at_t_end": l1,
                 "schedule": r32["schedule"], "host_compile_ms_per_step": r32["prof"]["host_compile_ms"] / args.steps,
                 "t_end_fp32": r32["t_end"], "t_end_fp64": r64["t_end"], "ms_per_step": r32["ms"] / args.steps,
                 "host_ms_per_step": (r32["prof"]["host_compile_ms"] + r32["prof"]["host_admesh_ms"]) / args.steps,
                 "wait_ms_per_step": r32["prof"]["wait_ms"] / args.steps,
                 "host_capture_ms_per_step": r32["prof"]["host_capture_ms"] / args.steps,
                 "step_gpu_ms_per_step": r32["prof"]["step_gpu_ms"] / args.steps},
        "host_ms_per_step": (prof["host_compile_ms"] + prof["host_admesh_ms"]) / args.steps,
        "rotor_batch": None if "rotor_batch" not in res else {
            "workload": "%d copies of the bench rotor in one handle (one launch per kernel over all their leaf "
                        "blocks), from t=%.2f; each copy is bit-identical to a single run, so the FP32 density "
                        "error is the fp32 entry's" % (ROTOR_BATCH, T0),
            "fp64": res["rotor_batch"]["fp64"], "fp32": res["rotor_batch"]["fp32"],
            "fp32_batched_vs_plain_fp64": res["rotor_batch"]["fp32"]["value"] / value,
            "l1_rel_density_vs_fp64_at_t_end": l1,
            "l2": "no flush: the 64 states (~0.5 GB FP32, ~1 GB FP64) exceed the 129 MB L2"},
        "batch": None if "batch" not in res else {
            "workload": "%d seeded cylindrical blasts (seed %d, amr_config_blast): [0,1]^2, gamma 1.4, 4 roots, "
                        "maxlevs U{3..6}, MUSCL-MC + HLLE + CT, CFL 0.2, outflow; %d untimed batch steps, then "
                        "%d timed" % (BATCH_N, BATCH_SEED, args.batch_advance, args.batch_steps),
            "fp64": res["batch"]["fp64"], "fp32": res["batch"]["fp32"],
            "fp32_two_handles_pipelined": res["batch"]["fp32_two_handles_pipelined"],
            "fp32_vs_plain_fp64_rotor": res["batch"]["fp32"]["value"] / value,
            "l1_rel_density_fp32_vs_fp64_max": res["batch"]["l1_rel_density_fp32_vs_fp64_max"],
            "l1_sample": "4 instances of the batch (maxlevs capped at 4) run to t = 0.1, finest uniform grid",
            "l2": "no flush: the 512 states (several GB) exceed the 129 MB L2"},
        "adjoint": None if "adjoint" not in res else dict(
            workload="Kelvin-Helmholtz, frozen 256^2 periodic mesh (256 blocks), gamma 5/3, MUSCL-MC + RUSA + CT, "
                     "RK2, 200 steps of dt 2e-4, loss = total density in [0.4,0.6]^2, gradient w.r.t. the 16 "
                     "amplitudes (seed %d); cost ratio = adjoint incl. recompute / plain forward, per step; "
                     "fd = central differences h = 1e-7 (first-order error from MC kinks); ke_loss: the same for "
                     "the transverse kinetic energy, a loss that scales with the perturbation" % KH_SEED,
            **res["adjoint"]),
        "orszag_tang": None if "orszag_tang" not in res else {
            "workload": "Orszag-Tang on [0,2pi]^2, periodic, 4x4 roots, gamma 5/3, HLLD + CT, RK2, to t=pi on a fixed "
                        "dt shared by both precisions; FP32 bulk vs FP64, relative L1 per conserved variable on the "
                        "finest uniform grid.  Reduced levels: with WENO5 the reference scheme (reproduced bit for "
                        "bit) loses pressure positivity at t~1.45 from 4 levels on",
            "runs": res["orszag_tang"]},
        "cpu_baseline": cpu,
        "clocks": {"sm_mhz": clk.get("sm_mhz"), "sm_max_mhz": clk.get("sm_max_mhz"), "reasons": clk.get("reasons", [])},
        "gpu_launches": int(prof["launches"]),
        "launches_per_step": round(int(prof["launches"]) / max(int(prof["steps"]), 1), 2),
    }
    print(json.dumps(line))
    return 0


if __name__ == "__main__":
    sys.exit(main())
