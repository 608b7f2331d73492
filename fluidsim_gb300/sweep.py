"""Sweeps of the 2D argon DC glow: many independent discharges of uneven grid
sizes (the voltage / pressure runs behind the reference's I-V curves,
plot-idvd.py), advanced together by the library's batch driver, and a small
autotuner that picks the multigrid smoother schedule per grid size.

The autotuner picks, per grid size, the multigrid smoother schedule (pre-
and post-sweeps per level) and the tile shape of the RK stage kernel.

Workload: `count` discharges with grid sizes drawn uniformly from SIZES
(squared), cathode voltage uniform in 150-400 V, pressure log-uniform in
0.5-10 Torr and secondary-emission coefficient uniform in 0.03-0.12, each from
its own seeded Gaussian-blob initial state with 1% noise.
"""
import time

import numpy as np

from . import abi, api, config, grid

SIZES = (64, 96, 128, 192, 256, 384, 512)


def sweep_specs(count=192, seed=0):
    """The seeded draw of the sweep's instances: list of dicts."""
    rng = np.random.default_rng(seed)
    n = rng.choice(SIZES, size=count)
    v = rng.uniform(150.0, 400.0, size=count)
    p = np.exp(rng.uniform(np.log(0.5), np.log(10.0), size=count))
    g = rng.uniform(0.03, 0.12, size=count)
    return [dict(n=int(n[i]), volts=float(v[i]), p_torr=float(p[i]), gam=float(g[i]), seed=int(seed * 1000 + i))
            for i in range(count)]


def make_config(spec, precision=abi.FS_PREC_FP64, mg_smooth=2, rtol=1e-8):
    return config.glow(spec["n"], p_torr=spec["p_torr"], gam=spec["gam"], vl=-spec["volts"] / config.PH0,
                       lapl_rtol=rtol, lapl_maxit=500, precision=precision, mg_smooth=mg_smooth)


TILES = ((32, 8), (32, 4), (64, 4))


def make_discharges(specs, precision=abi.FS_PREC_FP64, schedule=None):
    """One context per spec; schedule maps grid size -> mg_smooth (default 2)
    or -> (mg_smooth, stage tile) (FP64 contexts)."""
    out = []
    for s in specs:
        choice = (schedule or {}).get(s["n"], 2)
        nu, tile = choice if isinstance(choice, tuple) else (choice, None)
        cfg = make_config(s, precision, nu)
        mesh = cfg.mesh()
        k = api.constants(cfg)
        st = grid.blob_state(mesh, k, noise=0.01, seed=s["seed"], vl=cfg.vl)
        d = api.Discharge(cfg, mesh, st)
        if tile is not None and precision == abi.FS_PREC_FP64:
            d.set_stage_tile(*tile)
        out.append(d)
    return out


def run(discharges, steps, nthreads, warm=3, fused=False):
    """Warm up (start-up iterations and `warm` steps, untimed), then time
    `steps` main-loop iterations of every discharge with `nthreads` host
    threads (fused: the RK stages of all discharges as one launch per stage).
    Returns (aggregate steps/s, seconds, stats, return codes)."""
    api.batch_run(discharges, 2 + warm, nthreads=nthreads, check=False, fused=fused)
    t0 = time.perf_counter()
    stats, rcs = api.batch_run(discharges, steps, nthreads=nthreads, check=False, fused=fused)
    el = time.perf_counter() - t0
    ok = sum(1 for r in rcs if r == 0)
    return ok * steps / el, el, stats, rcs


def close(discharges):
    for d in discharges:
        d.close()


def autotune(specs, precision=abi.FS_PREC_FP64, candidates=(1, 2, 3), tiles=TILES, per_size=4, steps=6,
             nthreads=32):
    """For every grid size in specs, time up to `per_size` of its instances
    with each smoother schedule (mg_smooth = pre- and post-sweeps per level)
    and, on the FP64 path, each RK stage tile shape, and keep the fastest
    pair.  Returns ({size: (mg_smooth, tile)}, {size: {"nu/WxH": steps/s}})."""
    if precision != abi.FS_PREC_FP64:
        tiles = (None,)
    choice, table = {}, {}
    for n in sorted({s["n"] for s in specs}):
        sub = [s for s in specs if s["n"] == n][:per_size]
        table[n], best = {}, None
        for nu in candidates:
            for tile in tiles:
                ds = make_discharges(sub, precision, {n: (nu, tile)})
                try:
                    rate, _, _, rcs = run(ds, steps, nthreads, warm=2)
                    rate = rate if all(r == 0 for r in rcs) else 0.0
                finally:
                    close(ds)
                key = "%d/%s" % (nu, "x".join(map(str, tile)) if tile else "-")
                table[n][key] = rate
                if best is None or rate > best[0]:
                    best = (rate, (nu, tile))
        choice[n] = best[1]
    return choice, table
