"""Helpers of the GPU-vs-oracle parity tests."""
import numpy as np

from oracle import pyoracle as P


def run_pair(gpu_mod, steps, check_every=1, **cfg):
    """Advance the CUDA path and the oracle side by side; return per-step records.

    cfg uses the oracle's keywords (ic, limiter, flux, cfl, maxlevs, nghosts,
    nroots, periodic, geom_ref, gamma, tend, ic_param).
    """
    o = P.Oracle(**cfg).init()
    g = gpu_mod.Simulation(**to_gpu_cfg(cfg)).init()
    out = []
    for s in range(steps + 1):
        if s > 0:
            o.step()
            g.step()
        if s % check_every == 0 or s == steps:
            a, b = g.state(), o.state()
            same, dU, rel, dB = P.compare_states(a, b, cfg.get("nghosts", 2))
            full = same and np.array_equal(a["U"], b["U"]) and np.array_equal(a["Bi"], b["Bi"])
            out.append(dict(step=s, same_tree=same, bitwise=full, dU=dU, rel=rel, dB=dB,
                            t_equal=a["t"] == b["t"], leaves=int(b["leafs"].sum())))
            if not same:
                break
    return out, o, g


def to_gpu_cfg(c):
    return dict(ic=c.get("ic", "BWx"), limiter=c.get("limiter", "MC"), flux=c.get("flux", "RUSA"),
                cfl=c.get("cfl", 0.4), maxlevs=c.get("maxlevs", 4), nghosts=c.get("nghosts", 2),
                nroots=c.get("nroots", (2, 2)), periodic=c.get("periodic", False),
                geometry=0 if c.get("geom_ref", True) else 1, gamma=c.get("gamma", 0.0),
                t_end=c.get("tend", 0.0), ic_param=c.get("ic_param"),
                precision=c.get("precision", "fp64"), lenx=c.get("lenx", 1.0), leny=c.get("leny", 1.0),
                ct_type=c.get("ct_type", 1), diffusion=c.get("diffusion", False))


def oracle_kw(c, nthreads=8):
    """Oracle keyword arguments for a library configuration (amr_config)."""
    return dict(ic=c.ic.decode(), limiter=c.limiter.decode(), flux=c.flux.decode(), cfl=c.cfl,
                maxlevs=c.maxlevs, nghosts=c.nghosts, nroots=(c.nroots_x, c.nroots_y),
                periodic=bool(c.periodic), geom_ref=c.geometry == 0, gamma=c.gamma, tend=c.t_end,
                ic_param=list(c.ic_param), nthreads=nthreads, dt_fixed=c.dt_fixed, ct_type=c.ct_type or 1,
                diffusion=bool(c.diffusion))
