"""Benchmark of the fluidsim hot path on one GB300 (or N independent replicas).

Metric: steps/s of the 2D argon DC glow at 1024x1024 nodes -- one step is one
iteration of the reference's main loop (main.F90:68-121): ptcl_step with all
of its RK-Merson attempts, then lapl_solve (Poisson to 1e-8 relative residual),
then the accept/reject rotation.  Synthetic seeded inputs (Gaussian blob plus
1% noise, the workload's own definition; no dataset is involved).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--n 1024]
                  [--impl gb300|reference] [--dt adaptive|fixed]

The gb300 arm prints one JSON line with the device-resident throughput
(`value`), the end-to-end throughput through the C ABI with host buffers
(`e2e`), a roofline object for the dominant kernel (the RK stage kernel),
the CPU oracle timed on the host cores (`cpu_baseline`), SM clocks sampled
during the timed region and the number of kernels launched.  `value` and
`e2e` are the plain FP64 path (the drop-in); `variants` holds the same two
numbers for the mixed-precision solver and for the mixed solver with the
learned Poisson preconditioner (trained first on pairs harvested from the
run), each with its speed-up over the plain path, all at the same 1e-8
relative Poisson residual.

The reference arm (--impl reference) times the reference algorithm's CPU
implementation -- the C++ oracle, a restatement of the Fortran, because the
Fortran/MPI/PETSc reference cannot be built on this machine -- on all host
cores, on the same workload, a bounded number of steps.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)
# before anything creates the CUDA context (see fluidsim_gb300/__init__.py)
os.environ.setdefault("CUDA_DEVICE_MAX_CONNECTIONS", "32")

METRIC = "steps/s, 1024² glow: plain FP64 vs mixed+learned-PC at 1e-8 Poisson resid"
UNIT = "steps/s"
# FP64 algorithmic bytes of one RK stage launch per interior node:
# one RK-Merson attempt moves (25 S + 5) * 8 bytes per node with S = 3 species
# (stage 1 reads n2, n3, phi and writes k1, n2'; ...; stage 5 reads n2, n3,
# k1, k3, k4, phi and writes n1), i.e. 640 B per node per attempt, 128 B per stage.
STAGE_BYTES_PER_NODE = (25 * 3 + 5) * 8 / 5.0
# One FP64 stage launch on the 1024^2 workload, averaged over the five stages
# of an attempt, from one ncu capture (profiles/k_stage_glow1024.md):
# DRAM traffic (dram__bytes_read.sum + dram__bytes_write.sum) per launch,
STAGE_TRAFFIC_1024 = 167.2e6
# FP64 work per interior node, flops = dadd + dmul + 2 dfma
# (sm__sass_thread_inst_executed_op_{dadd,dmul,dfma}_pred_on.sum / nodes),
STAGE_FP64_FLOPS_PER_NODE = 297.2
# and FP64-pipe thread instructions per node (sm__inst_executed_pipe_fp64.sum
# x 32 / nodes: the DFMA/DADD/DMUL above plus conversions and comparisons),
# the resource the kernel's time is bound by
STAGE_FP64_PIPE_INST_PER_NODE = 245.0
# algorithmic HBM bytes per node of one step's parts (FP64, 3 species): an RK
# attempt (640), the Poisson assembly (reads n_e, n_i, n_t, phi; writes b and
# three operator fields: 64) and one multigrid-PCG iteration (~57 fields: 456)
STEP_ATTEMPT_BYTES = 640
STEP_ASSEMBLY_BYTES = 64
STEP_CG_BYTES = 456
# learned preconditioner variant: training pairs harvested over LPC_HARVEST
# steps (4 per step: full 1024^2 grids), then LPC_ITERS Adam steps (lr 1e-3)
# on batches of LPC_BATCH random 128 x 128 crops
# the device control block the host reads once per RK attempt and twice per
# Poisson solve (sizeof(Ctrl) in fluidsim_gb300/csrc/fs_internal.h)
CTRL_BYTES = 312
LPC_HARVEST = 12
LPC_ITERS = 2000
LPC_BATCH = 64
LPC_FORCED_STEPS = 20


def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return d.get("hbm_gbs", 6800.0), "measured"
    return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.f = None

    def start(self):
        self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.Q,
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=self.f, stderr=subprocess.DEVNULL)
        except (FileNotFoundError, OSError):
            self.proc = None

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        self.proc.wait()
        self.f.flush()
        self.f.seek(0)
        rows = [r.split(",") for r in self.f.read().strip().splitlines() if r.strip()]
        os.unlink(self.f.name)
        sm, smax, reasons = [], [], set()
        names = ("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap")
        for r in rows:
            try:
                sm.append(float(r[1]))
                smax.append(float(r[2]))
            except (ValueError, IndexError):
                continue
            for n, v in zip(names, r[5:9]):
                if v.strip().lower() == "active":
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def workload(n, dt_mode, rtol=1e-8, precision="fp64"):
    from fluidsim_gb300 import abi, config
    cfg = config.glow(n, adaptive=1 if dt_mode == "adaptive" else 0, lapl_rtol=rtol,
                      lapl_maxit=500,
                      precision=abi.FS_PREC_MIXED if precision == "mixed" else abi.FS_PREC_FP64)
    return cfg


def initial_state(cfg, mesh, k):
    from fluidsim_gb300 import grid
    return grid.blob_state(mesh, k, noise=0.01, seed=1, vl=cfg.vl)


def cpu_threads():
    try:
        return len(os.sched_getaffinity(0))
    except AttributeError:
        return os.cpu_count() or 1


def time_oracle(cfg, mesh, state, t, dt, ts, max_seconds, max_steps, threads):
    """Run the oracle from a given state; returns (steps, seconds)."""
    from oracle import oracle
    oracle.set_threads(threads, timed=True)
    o = oracle.OracleDischarge(cfg, mesh, state, solver=oracle.SOLVER_BICGSTAB, timed=True)
    o.set_time(t, dt)
    o.ts = ts
    steps = 0
    t0 = time.perf_counter()
    while steps < max_steps:
        o.step()
        steps += 1
        if time.perf_counter() - t0 > max_seconds:
            break
    el = time.perf_counter() - t0
    o.close()
    return steps, el


def run_reference(args):
    """--impl reference: the reference algorithm's CPU implementation."""
    ws, rank, _ = dist_env()
    if rank != 0:
        return 0
    from fluidsim_gb300 import api
    from oracle import oracle
    oracle.build()
    cfg = workload(args.n, args.dt)
    mesh = cfg.mesh()
    k = api.constants(cfg, oracle.load(timed=True), "or_")
    st = initial_state(cfg, mesh, k)
    threads = cpu_threads()
    oracle.set_threads(threads, timed=True)
    o = oracle.OracleDischarge(cfg, mesh, st, solver=oracle.SOLVER_BICGSTAB, timed=True)
    # start-up iterations (Poisson only) and the requested warm-up steps,
    # untimed; the warm-up stops early only past 30 s (a step takes ~1.7 s
    # at 1024^2 on 16 cores), and the line reports the count run
    for _ in range(2):
        o.step()
    warm = 0
    tw = time.perf_counter()
    while warm < args.warmup and (warm < 3 or time.perf_counter() - tw < 30.0):
        o.step()
        warm += 1
    budget = float(os.environ.get("FS_REF_BUDGET_S", "60"))
    steps = 0
    t0 = time.perf_counter()
    while steps < args.steps:
        o.step()
        steps += 1
        if time.perf_counter() - t0 > budget:
            break
    el = time.perf_counter() - t0
    v = steps / el
    line = {
        "impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": ws,
        "steps": steps, "warmup": warm, "ms_per_step": 1e3 * el / steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic: seeded Gaussian blob + 1% noise",
        "config": {"workload": "2D Ar DC glow %dx%d, %s dt, Poisson rtol 1e-8" % (args.n, args.n, args.dt),
                   "solver": "BiCGStab + block-Jacobi ILU(0), one block per thread",
                   "build": "C++ oracle, g++ -O3 -fopenmp -ffp-contract=fast"},
        "cpu_baseline": {"value": v, "unit": UNIT, "cores": threads, "kind": "port",
                         "sample": "%d main-loop steps of the same workload after start-up" % steps},
        "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))
    return 0


def measure_variant(cfg, mesh, st0, args, barrier, target_ts, learned=False):
    """Device-resident and end-to-end steps/s of one solver variant on the
    same workload (fresh context, same warm-up), for the comparison keys.
    learned: first harvest training pairs from the plain multigrid-PCG over
    LPC_HARVEST steps, train the network (LPC_ITERS Adam steps), then time
    with the network in the solver."""
    import torch
    from fluidsim_gb300 import api
    d = api.Discharge(cfg, mesh, st0)
    stream = torch.cuda.ExternalStream(d.stream_handle())
    d.run(target_ts)               # the plain run's checkpoint step
    train = None
    if learned:
        t0 = time.perf_counter()
        d.lpc_init(crop=128, max_batch=LPC_BATCH, max_samples=4 * LPC_HARVEST, seed=1)
        for _ in range(LPC_HARVEST):
            d.step()
            d.lpc_harvest(per_solve=4)
        hist = d.lpc_train(iters=LPC_ITERS, batch=LPC_BATCH, lr=1e-3, seed=2)
        d.lpc_use(True)
        # warm-up with the network in the loop: its CUDA graph is built and the
        # solver's judge takes its first measurements of both solvers
        d.run(args.warmup)
        torch.cuda.synchronize()
        train = {"pairs": d.lpc_info()["samples"], "adam_steps": LPC_ITERS, "batch": LPC_BATCH,
                 "crop": 128, "crops_seen": LPC_ITERS * LPC_BATCH,
                 "loss_first20": float(hist[:20].mean()), "loss_last20": float(hist[-20:].mean()),
                 "seconds": time.perf_counter() - t0, "nn_grid": [d.lpc_info()["h"], d.lpc_info()["w"]],
                 "params": d.lpc_info()["nparam"]}
    warm_state = d.download(nlev=3)
    warm_t, warm_dt, warm_ts = d.t, d.dt, d.ts
    w = d.stats()
    li0 = d.lpc_info() if learned else None
    l0 = d.launch_count()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    barrier()
    torch.cuda.synchronize()
    e0.record(stream)
    s = d.run(args.steps)
    e1.record(stream)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1)
    launches = d.launch_count() - l0
    nn = None
    if learned:
        li1 = d.lpc_info()
        ns = li1["solves"] - li0["solves"]
        nn = {"timed_solves": ns, "with_network": li1["nn_solves"] - li0["nn_solves"],
              "fraction": (li1["nn_solves"] - li0["nn_solves"]) / max(ns, 1)}
    pinned = {}
    for key in ("ni", "ne", "nt", "ph"):
        t = torch.empty(warm_state[key].shape[::-1], dtype=torch.float64, pin_memory=True)
        v = t.numpy().T
        v[...] = warm_state[key]
        pinned[key] = v
    d.set_time(warm_t, warm_dt)
    d.ts = warm_ts
    barrier()
    torch.cuda.synchronize()
    out = {key: torch.empty(pinned[key].shape[::-1], dtype=torch.float64, pin_memory=True).numpy().T
           for key in ("ni", "ne", "nt", "ph")}
    a0 = d.stats()["attempts"]
    e2, e3 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e2.record(stream)
    d.upload(pinned)
    for _ in range(args.steps):
        d.step()
    d.download(nlev=3, out=out)   # straight into pinned host memory
    e3.record(stream)
    torch.cuda.synchronize()
    ms_e2e = e2.elapsed_time(e3)
    e2e_attempts = d.stats()["attempts"] - a0
    off = d.lpc_info()["off"] if learned else None
    forced = None
    if learned:
        # the network in every solve (mode 2), from the same state: what the
        # judge weighs against the plain solver
        d.upload(pinned)
        d.set_time(warm_t, warm_dt)
        d.ts = warm_ts
        d.lpc_use(2)
        d.run(2)
        f0 = d.stats()
        e4, e5 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        e4.record(stream)
        f1 = d.run(LPC_FORCED_STEPS)
        e5.record(stream)
        torch.cuda.synchronize()
        nst = f1["steps"] - f0["steps"]
        forced = {"steps": nst, "ms_per_step": e4.elapsed_time(e5) / max(nst, 1),
                  "cg_iters_per_step": (f1["lapl_iters"] - f0["lapl_iters"]) / max(nst, 1),
                  "network_switched_off_in_last_solve": d.lpc_info()["off"]}
    d.close()
    return {"value": args.steps / (ms * 1e-3), "ms_per_step": ms / args.steps,
            "e2e": args.steps / (ms_e2e * 1e-3),
            "cg_iters_per_step": (s["lapl_iters"] - w["lapl_iters"]) / args.steps,
            "rk_attempts": s["attempts"] - w["attempts"], "gpu_launches": launches,
            "h2d_bytes_per_step": (sum(a.nbytes for a in pinned.values()) + 8 * args.steps) / args.steps,
            "d2h_bytes_per_step": (sum(a.nbytes for a in out.values())
                                   + CTRL_BYTES * (e2e_attempts + 2 * args.steps)) / args.steps,
            "training": train, "network_use": nn, "network_switched_off_in_last_solve": off,
            "network_every_solve": forced}


def run_accuracy(args):
    """--accuracy: per-field error of the mixed-precision path against the FP64
    path after `acc_steps` adaptive steps of the workload.  The FP64 run
    replays the mixed run's accepted step sizes with the controller off, so
    both integrate the same step sequence (two adaptive runs choose slightly
    different dt and drift apart in time); the FP64 GPU path matches the CPU
    oracle to 1e-10 (64x64: 4e-14 after 2000 fixed-dt steps)."""
    import numpy as np
    import torch
    torch.cuda.set_device(0)
    import __graft_entry__
    __graft_entry__.build()
    from fluidsim_gb300 import abi, api
    cfg = workload(args.n, "adaptive")
    cfgm = workload(args.n, "adaptive", precision="mixed")
    mesh = cfg.mesh()
    k = api.constants(cfg)
    st = initial_state(cfg, mesh, k)
    a = api.Discharge(cfg.replace(adaptive=0), mesh, st)
    b = api.Discharge(cfgm, mesh, st)

    def errs(gm, gf):
        out = {}
        for f in ("ni", "ne", "nt"):
            x, y = np.asarray(gm[f])[1:-1, 1:-1], np.asarray(gf[f])[1:-1, 1:-1]
            out[f] = {"linf_rel": float(np.max(np.abs(x - y) / (np.abs(y) + k["n_zero"]))),
                      "l2_rel": float(np.linalg.norm(x - y) / np.linalg.norm(y))}
        x, y = np.asarray(gm["ph"])[1:-1, 1:-1], np.asarray(gf["ph"])[1:-1, 1:-1]
        out["ph"] = {"linf_rel": float(np.max(np.abs(x - y)) / np.max(np.abs(y))),
                     "l2_rel": float(np.linalg.norm(x - y) / np.linalg.norm(y))}
        return out

    marks = sorted({m for m in (10, 100, 500, 1000, args.acc_steps) if m <= args.acc_steps})
    rows = []
    max_relres = 0.0
    for s in range(1, args.acc_steps + 1):
        gb = b.step()
        if gb["lerr"]:
            raise RuntimeError("mixed Poisson solve failed at step %d" % s)
        max_relres = max(max_relres, gb["relres"])
        if a.ts > 1:
            a.dt = b.stats()["dt_step"]
            a.ptcl_step()
        a.dt = b.dt
        if a.lapl_solve()["lerr"]:
            raise RuntimeError("FP64 Poisson solve failed at step %d" % s)
        a.accept()
        if s in marks:
            rows.append({"step": s, "t_s": b.t * 1e-6, "errors": errs(b.download(), a.download())})
    line = {"metric": "per-field relative error, mixed vs FP64, %dx%d glow" % (args.n, args.n),
            "steps": args.acc_steps, "max_mixed_relres": max_relres, "poisson_rtol": cfg.lapl_rtol,
            "checkpoints": rows}
    print(json.dumps(line))
    return 0


def run_sweep(args):
    """--sweep: the batched uneven sweep.  Aggregate steps/s of `sweep_count`
    independent discharges (grid sizes 64..512 squared, voltage, pressure and
    gamma drawn from a seed), each advanced `sweep_steps` main-loop iterations:
    one after another (the sequential baseline), all together through the
    batch driver with the fixed smoother schedule, and all together with the
    schedule the autotuner picks per grid size."""
    import torch
    torch.cuda.set_device(0)
    import __graft_entry__
    __graft_entry__.build()
    from fluidsim_gb300 import abi, sweep
    specs = sweep.sweep_specs(args.sweep_count, seed=0)
    res = {}
    t0 = time.perf_counter()
    choice, table = sweep.autotune(specs, abi.FS_PREC_FP64, nthreads=args.sweep_threads)
    t_tune = time.perf_counter() - t0
    for name, threads, sched, fused in (("sequential_fixed", 1, None, False),
                                        ("batched_fixed", args.sweep_threads, None, False),
                                        ("batched_autotuned", args.sweep_threads, choice, False),
                                        ("fused_autotuned", args.sweep_threads, choice, True)):
        ds = sweep.make_discharges(specs, abi.FS_PREC_FP64, sched)
        try:
            rate, el, stats, rcs = sweep.run(ds, args.sweep_steps, threads, fused=fused)
            # electron inventory per discharge (after the timed region): a
            # fingerprint of every instance's state, compared across drivers
            ne_sum = [float(d.download()["ne"][1:-1, 1:-1].sum()) for d in ds]
        finally:
            sweep.close(ds)
        res[name] = {"steps_per_s": rate, "seconds": el, "failed": [i for i, r in enumerate(rcs) if r != 0],
                     "rk_rejects": sum(s["rk_rejects"] for s in stats),
                     "idc": [s["idc"] for s in stats], "ida": [s["ida"] for s in stats],
                     "t_end_s": [s["t"] * 1e-6 for s in stats], "ne_sum": ne_sum}
    line = {
        "metric": "aggregate steps/s, %d-discharge uneven sweep (grids 64-512^2)" % args.sweep_count,
        "value": max(res["batched_autotuned"]["steps_per_s"], res["fused_autotuned"]["steps_per_s"]),
        "driver": ("fused" if res["fused_autotuned"]["steps_per_s"] >= res["batched_autotuned"]["steps_per_s"]
                   else "concurrent contexts"),
        "unit": UNIT, "n_gpus": 1,
        "steps": args.sweep_steps, "higher_is_better": True, "scaling": "strong", "vs_baseline": None,
        "dtype": "f64", "data": "synthetic: seeded sweep of V ~ U(150,400) V, p ~ logU(0.5,10) Torr, "
                                "gamma ~ U(0.03,0.12), Gaussian-blob initial states",
        "config": {"workload": "batched uneven sweep", "instances": args.sweep_count,
                   "steps_per_instance": args.sweep_steps, "host_threads": args.sweep_threads,
                   "sizes": {str(n): sum(1 for s in specs if s["n"] == n) for n in sweep.SIZES}},
        "runs": res,
        "speedup_batched_autotuned_vs_sequential": res["batched_autotuned"]["steps_per_s"]
                                                   / res["sequential_fixed"]["steps_per_s"],
        "speedup_fused_vs_sequential": res["fused_autotuned"]["steps_per_s"] / res["sequential_fixed"]["steps_per_s"],
        "speedup_fused_vs_batched": res["fused_autotuned"]["steps_per_s"] / res["batched_autotuned"]["steps_per_s"],
        "fused_idc_equals_batched": res["fused_autotuned"]["idc"] == res["batched_autotuned"]["idc"],
        "fused_state_equals_batched": (res["fused_autotuned"]["ne_sum"] == res["batched_autotuned"]["ne_sum"]
                                       and res["fused_autotuned"]["t_end_s"] == res["batched_autotuned"]["t_end_s"]),
        "speedup_autotuned_vs_fixed": res["batched_autotuned"]["steps_per_s"]
                                      / res["batched_fixed"]["steps_per_s"],
        "autotune": {"mg_smooth_and_stage_tile_by_size": {str(k): [v[0], list(v[1]) if v[1] else None]
                                                          for k, v in choice.items()},
                     "steps_per_s_by_size": {str(k): dict(v) for k, v in table.items()},
                     "seconds": t_tune},
    }
    print(json.dumps(line))
    return 0


def timed_steps(d, steps, stream, barrier, ws):
    """Device-resident main-loop steps timed with CUDA events on the context's
    stream, max over ranks.  Returns (ms, stats after, launches)."""
    import torch
    l0 = d.launch_count()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    barrier()
    torch.cuda.synchronize()
    e0.record(stream)
    s = d.run(steps)
    e1.record(stream)
    torch.cuda.synchronize()
    barrier()
    ms = e0.elapsed_time(e1)
    if ws > 1:
        import torch.distributed as dist
        t = torch.tensor([ms], device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms = float(t.item())
    return ms, s, d.launch_count() - l0


def fp64_peak_tflops(device):
    """FP64 roof of this GPU, measured now: 2 x the DFMA rate of the library's
    own microbenchmark (fs_fp64_rate; CUDA events, no clock changes)."""
    import ctypes as C
    from fluidsim_gb300 import api
    v = C.c_double()
    rc = api.load_library().fs_fp64_rate(int(device), C.byref(v))
    if rc != 0:
        raise RuntimeError("fs_fp64_rate failed (%d)" % rc)
    return 2.0 * v.value / 1e12


def run_gpu(args):
    import numpy as np
    import torch
    ws, rank, local = dist_env()
    if ws > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    else:
        torch.cuda.set_device(0)
    import __graft_entry__
    __graft_entry__.build()
    from fluidsim_gb300 import api
    torch.cuda.init()

    cfg = workload(args.n, args.dt, precision=args.precision)
    mesh = cfg.mesh()
    k = api.constants(cfg)
    st0 = initial_state(cfg, mesh, k)
    d = api.Discharge(cfg, mesh, st0)
    stream = torch.cuda.ExternalStream(d.stream_handle())

    def barrier():
        if ws > 1:
            import torch.distributed as dist
            dist.barrier()

    # ---- start-up figure: right after the two Poisson-only iterations -------
    d.run(2 + args.warmup)
    w0 = d.stats()
    ms0, s0, _ = timed_steps(d, args.steps, stream, barrier, ws)
    startup = {"value": ws * args.steps / (ms0 * 1e-3), "ms_per_step": ms0 / args.steps,
               "from_step": w0["steps"], "rk_attempts": s0["attempts"] - w0["attempts"],
               "rk_rejects": s0["rk_rejects"] - w0["rk_rejects"],
               "cg_iters_per_step": (s0["lapl_iters"] - w0["lapl_iters"]) / args.steps}

    # ---- developed state: checkpoint after >= args.develop adaptive steps ----
    more = max(0, args.develop - d.ts)
    if more:
        d.run(more)
    d.run(args.warmup)
    ck = d.checkpoint()
    warm_stats = d.stats()

    # ---- timed region: device-resident steps from the checkpoint ------------
    sampler = ClockSampler(local)
    sampler.start()
    d.profile(["stage"])          # CUDA events around the RK stage launches only
    ms, s, launches = timed_steps(d, args.steps, stream, barrier, ws)
    clocks = sampler.stop()
    prof = d.profile_read()
    d.profile([])
    attempts = s["attempts"] - warm_stats["attempts"]
    rejects = s["rk_rejects"] - warm_stats["rk_rejects"]
    iters = s["lapl_iters"] - warm_stats["lapl_iters"]

    # ---- end to end through the C ABI with host buffers ---------------------
    pinned = {}
    for key in ("ni", "ne", "nt", "ph"):
        a = ck["state"][key]
        t = torch.empty(a.shape[::-1], dtype=torch.float64, pin_memory=True)
        v = t.numpy().T          # Fortran-ordered view of pinned memory
        v[...] = a
        pinned[key] = v
    out = {key: torch.empty(pinned[key].shape[::-1], dtype=torch.float64, pin_memory=True).numpy().T
           for key in ("ni", "ne", "nt", "ph")}
    state_bytes = sum(a.nbytes for a in pinned.values())
    d.restore(ck)               # time, dt, controller, circuit (untimed)
    d.ts = ck["controller"]["ts"]
    a0 = d.stats()["attempts"]
    barrier()
    torch.cuda.synchronize()
    e2, e3 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e2.record(stream)
    d.upload(pinned)
    for _ in range(args.steps):
        d.step()                  # fs_ptcl_step + fs_lapl_solve + fs_accept/fs_reject
    d.download(nlev=3, out=out)   # straight into pinned host memory
    e3.record(stream)
    torch.cuda.synchronize()
    barrier()
    ms_e2e = e2.elapsed_time(e3)
    e2e_attempts = d.stats()["attempts"] - a0
    if ws > 1:
        import torch.distributed as dist
        t = torch.tensor([ms_e2e], device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms_e2e = float(t.item())

    # ---- per-class kernel time on a separate pass (Krylov loop host-driven) --
    d.restore(ck)
    d.ts = ck["controller"]["ts"]
    d.profile(None)
    d.run(args.steps)
    breakdown = d.profile_read()
    d.profile([])

    # ---- optional: the reference's output files every K steps ---------------
    # The same steps from the checkpoint with and without a record (the
    # writeOut files) after every K steps; the writer thread's last record is
    # on disk before the closing event.
    output = None
    if args.output_every > 0:
        K = args.output_every
        res = {}
        with tempfile.TemporaryDirectory() as td:
            for write in (False, True):
                d.restore(ck)
                d.ts = ck["controller"]["ts"]
                if write:
                    d.write_output(td, init=True)
                    d.output_wait()
                barrier()
                torch.cuda.synchronize()
                e4, e5 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                call_s, done = 0.0, 0
                e4.record(stream)
                while done < args.steps:
                    n = min(K, args.steps - done)
                    d.run(n)
                    done += n
                    if write:
                        t0 = time.perf_counter()
                        d.write_output(td)
                        call_s += time.perf_counter() - t0
                if write:
                    d.output_wait()
                e5.record(stream)
                torch.cuda.synchronize()
                res[write] = (e4.elapsed_time(e5), call_s)
        nrec = (args.steps + K - 1) // K
        output = {"every": K, "records": nrec,
                  "steps_per_s_without": args.steps / (res[False][0] * 1e-3),
                  "steps_per_s_with": args.steps / (res[True][0] * 1e-3),
                  "call_ms": 1e3 * res[True][1] / nrec}

    # ---- roofline of the dominant kernel (RK stage, FP64-issue-bound) -------
    hbm_peak, peak_kind = measured_peaks()
    fp64_peak = fp64_peak_tflops(local)
    st_ms, st_n = prof["stage"]
    nodes = cfg.nx * cfg.ny
    stage_ms = st_ms / max(st_n, 1)
    fp64_achieved = STAGE_FP64_FLOPS_PER_NODE * nodes / (stage_ms * 1e-3) / 1e12
    pipe_achieved = STAGE_FP64_PIPE_INST_PER_NODE * nodes / (stage_ms * 1e-3) / 1e9
    hbm_achieved = STAGE_BYTES_PER_NODE * nodes / (stage_ms * 1e-3) / 1e9
    # DRAM bytes of one stage launch (dram__bytes_read.sum + dram__bytes_write.sum)
    # from one ncu capture of the 1024^2 workload; scaled by nodes elsewhere
    traffic = STAGE_TRAFFIC_1024 * nodes / (1024.0 * 1024.0)
    # the whole step against HBM: algorithmic bytes of the RK attempts, the
    # assembly and the CG iterations actually run
    step_bytes = (STEP_ATTEMPT_BYTES * attempts + STEP_ASSEMBLY_BYTES * args.steps
                  + STEP_CG_BYTES * iters) * nodes / args.steps
    step_gbs = step_bytes / (ms / args.steps * 1e-3) / 1e9

    # ---- CPU baseline: the oracle on the host cores, bounded sample ---------
    cpu = None
    if rank == 0 and not args.no_cpu:
        threads = cpu_threads()
        steps_c, el_c = time_oracle(cfg, mesh, ck["state"], ck["t"], ck["dt"], ck["controller"]["ts"],
                                    max_seconds=args.cpu_seconds, max_steps=args.steps, threads=threads)
        cpu = {"value": steps_c / el_c, "unit": UNIT, "cores": threads, "kind": "port",
               "sample": "%d main-loop steps of the %dx%d workload from the same checkpoint "
                         "(C++ oracle built -O3 with OpenMP, BiCGStab+ILU(0))" % (steps_c, args.n, args.n)}

    # ---- the mixed-precision solver on the same workload ---------------------
    variants = {}
    if args.precision == "fp64" and not args.no_variants:
        cfgm = workload(args.n, args.dt, precision="mixed")
        vm = measure_variant(cfgm, mesh, st0, args, barrier, ck["controller"]["ts"])
        vm["speedup_vs_plain"] = vm["value"] / (args.steps / (ms * 1e-3))
        vm["e2e_speedup_vs_plain"] = vm["e2e"] / (args.steps / (ms_e2e * 1e-3))
        variants["mixed"] = vm
        vl = measure_variant(cfgm, mesh, st0, args, barrier, ck["controller"]["ts"], learned=True)
        vl["speedup_vs_plain"] = vl["value"] / (args.steps / (ms * 1e-3))
        vl["e2e_speedup_vs_plain"] = vl["e2e"] / (args.steps / (ms_e2e * 1e-3))
        variants["mixed+learned-PC"] = vl

    if rank == 0:
        total_ms = {kk: v[0] for kk, v in breakdown.items()}
        line = {
            "metric": METRIC, "value": ws * args.steps / (ms * 1e-3), "unit": UNIT, "n_gpus": ws,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic: seeded Gaussian blob (1e14 m^-3, sigma 1 mm) + 1% noise",
            "config": {"workload": "2D Ar DC glow %dx%d, plain FP64 path" % (args.n, args.n),
                       "dt": args.dt, "poisson_rtol": 1e-8, "species": 3,
                       "timed_from_step": ck["controller"]["ts"],
                       "rk_attempts": attempts, "rk_rejects": rejects,
                       "cg_iters_per_step": iters / args.steps,
                       "l2": "working set per step > 129 MB L2 (no flush needed)",
                       "parallelism": "replicas" if ws > 1 else "single GPU"},
            "startup": startup,
            "e2e": {"value": ws * args.steps / (ms_e2e * 1e-3), "unit": UNIT,
                    "h2d_bytes_per_step": (state_bytes + 8 * args.steps) / args.steps,
                    "d2h_bytes_per_step": (state_bytes + CTRL_BYTES * (e2e_attempts + 2 * args.steps)) / args.steps},
            "roofline": {"bound": "fp64", "achieved": fp64_achieved, "peak": fp64_peak, "unit": "TFLOP/s",
                         "frac": fp64_achieved / fp64_peak, "traffic": traffic,
                         "kernel": "k_stage (RK-Merson stage, FP64)",
                         "peak_kind": "measured in this run (fs_fp64_rate: 2 x DFMA/s)",
                         "flops_per_node": STAGE_FP64_FLOPS_PER_NODE, "stage_ms": stage_ms,
                         "fp64_pipe": {"achieved": pipe_achieved, "peak": fp64_peak / 2 * 1e3,
                                       "unit": "G inst/s", "frac": pipe_achieved / (fp64_peak / 2 * 1e3),
                                       "inst_per_node": STAGE_FP64_PIPE_INST_PER_NODE},
                         "hbm": {"achieved": hbm_achieved, "peak": hbm_peak, "unit": "GB/s",
                                 "frac": hbm_achieved / hbm_peak, "peak_kind": peak_kind,
                                 "bytes_per_node": STAGE_BYTES_PER_NODE},
                         "step_hbm": {"achieved": step_gbs, "peak": hbm_peak, "unit": "GB/s",
                                      "frac": step_gbs / hbm_peak, "bytes_per_step": step_bytes}},
            "kernel_ms_per_step": {kk: v / args.steps for kk, v in total_ms.items()},
            "cpu_baseline": cpu,
            "variants": variants,
            "clocks": clocks,
            "gpu_launches": launches,
        }
        if output is not None:
            line["output"] = output
        print(json.dumps(line))
    d.close()
    if ws > 1:
        import torch.distributed as dist
        dist.destroy_process_group()
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=100)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--n", type=int, default=1024)
    ap.add_argument("--impl", default="gb300", choices=("gb300", "reference"))
    ap.add_argument("--dt", default="adaptive", choices=("adaptive", "fixed"))
    ap.add_argument("--precision", default="fp64", choices=("fp64", "mixed"))
    ap.add_argument("--cpu-seconds", type=float, default=30.0)
    ap.add_argument("--develop", type=int, default=500,
                    help="main-loop steps run before the checkpoint the timed steps start from")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-variants", action="store_true",
                    help="skip the mixed-precision comparison run")
    ap.add_argument("--sweep", action="store_true", help="the batched uneven sweep instead")
    ap.add_argument("--output-every", type=int, default=0,
                    help="also time the steps with the reference's output files written every K steps")
    ap.add_argument("--accuracy", action="store_true",
                    help="per-field error of the mixed path against the FP64 path instead")
    ap.add_argument("--acc-steps", type=int, default=2000)
    ap.add_argument("--sweep-count", type=int, default=192)
    ap.add_argument("--sweep-steps", type=int, default=40)
    ap.add_argument("--sweep-threads", type=int, default=32)
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        return run_reference(args)
    if args.sweep:
        return run_sweep(args)
    if args.accuracy:
        return run_accuracy(args)
    return run_gpu(args)


if __name__ == "__main__":
    sys.exit(main())
