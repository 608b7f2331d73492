"""GPU path against the CPU oracle at the benchmark's own sizes (needs a GB300).

* 1024x1024, the benchmark workload itself (Gaussian blob, 1 % noise, seed 1,
  -250 V across the gap): the two Poisson-only start-up iterations and three
  full steps of the main loop (main.F90:68-121).  Poisson on both sides to a
  1e-14 relative residual (GPU multigrid-PCG; oracle BiCGStab with
  block-Jacobi ILU(0), the CPU solver PETSc would use by default).
* 256x256, 50 adaptive steps: identical RK attempt counts every step, fields
  compared along the way.
* 64x64 with the adaptive controller (rel tol 1e-4), 2000 steps: the
  accept/reject sequence is compared step by step and the first step at which
  it differs is reported; the fields are compared up to that step.

Per-field error: relative L-infinity over interior nodes with the density
floor n_zero as absolute guard; phi relative to max|phi|.  Every test prints
one JSON line with the errors it measured.
"""
import json
import os

import numpy as np
import pytest

from tests._util import field_errors

pytestmark = pytest.mark.gpu


def _threads():
    try:
        return len(os.sched_getaffinity(0))
    except AttributeError:
        return os.cpu_count() or 1


def _pair(n, seed, solver_rtol=1e-14, oracle_direct=False, **kw):
    from fluidsim_gb300 import api, config, grid
    from oracle import oracle
    cfg = config.glow(n, lapl_rtol=solver_rtol, lapl_maxit=2000, **kw)
    mesh = cfg.mesh()
    k = api.constants(cfg)
    st = grid.blob_state(mesh, k, noise=0.01, seed=seed, vl=cfg.vl)
    oracle.set_threads(_threads())
    gpu = api.Discharge(cfg, mesh, st)
    ocfg = cfg.replace(lapl_maxit=20000)
    solver = oracle.SOLVER_DIRECT if oracle_direct else oracle.SOLVER_BICGSTAB
    ref = oracle.OracleDischarge(ocfg, mesh, st, solver=solver)
    return cfg, mesh, k, st, gpu, ref


def _floor(cfg, mesh, k, st, nsteps, solver):
    """Oracle against itself on inputs perturbed by 1e-15 (relative): the
    rounding sensitivity of the run, the bar's floor where the run itself
    amplifies rounding."""
    from oracle import oracle
    rng = np.random.default_rng(0)
    st2 = {f: (np.asfortranarray(v * (1 + 1e-15 * rng.standard_normal(v.shape))) if f != "ph" else v)
           for f, v in st.items()}
    ocfg = cfg.replace(lapl_maxit=20000)
    a = oracle.OracleDischarge(ocfg, mesh, st, solver=solver)
    b = oracle.OracleDischarge(ocfg, mesh, st2, solver=solver)
    for _ in range(nsteps):
        a.step(), b.step()
    return field_errors(a.download(), b.download(), k["n_zero"])


def test_benchmark_workload_1024(built):
    """The 1024^2 workload every benchmark number is measured on: per field
    within 1e-10 after the first full step (or 10x the oracle's own rounding
    sensitivity where that is larger), and within 1e-9 after three."""
    from oracle import oracle
    cfg, mesh, k, st, gpu, ref = _pair(1024, seed=1)
    rec = {"grid": 1024, "steps": []}
    for s in range(5):                 # 2 Poisson-only start-up iterations, then 3 steps
        gi, ri = gpu.step(), ref.step()
        assert gi["lerr"] == 0 and ri["lerr"] == 0, (s, gi, ri)
        e = field_errors(gpu.download(), ref.download(), k["n_zero"])
        row = {"iter": s, "err": e, "gpu_iters": gi["iters"], "gpu_relres": gi["relres"],
               "oracle_iters": ri["iters"], "oracle_relres": ri["relres"]}
        if s >= 2:
            assert gi["attempts"] == ri["attempts"], (s, gi, ri)
            row["attempts"] = gi["attempts"]
            row["dt_rel"] = abs(gi["dt"] - ri["dt"]) / abs(ri["dt"])
        rec["steps"].append(row)
    print(json.dumps(rec))
    e1 = rec["steps"][2]["err"]
    if max(e1.values()) > 1e-10:
        fl = _floor(cfg, mesh, k, st, 3, oracle.SOLVER_BICGSTAB)
        rec["floor_after_step1"] = fl
        print(json.dumps({"floor_after_step1": fl}))
        for f in e1:
            assert e1[f] <= max(1e-10, 10 * fl[f]), (f, e1, fl)
    e3 = rec["steps"][4]["err"]
    assert max(e3.values()) <= 1e-9, e3


def test_adaptive_256_fifty_steps(built):
    """50 adaptive steps at 256^2: the same RK attempts every step and every
    field within 1e-9 of the oracle's throughout."""
    cfg, mesh, k, st, gpu, ref = _pair(256, seed=1)
    worst, attempts = {}, []
    for s in range(52):
        gi, ri = gpu.step(), ref.step()
        assert gi["lerr"] == 0 and ri["lerr"] == 0, (s, gi, ri)
        if s >= 2:
            assert gi["attempts"] == ri["attempts"], (s, gi, ri)
            attempts.append(gi["attempts"])
        if s % 10 == 1 or s == 51:
            e = field_errors(gpu.download(), ref.download(), k["n_zero"])
            worst = {f: max(worst.get(f, 0.0), v) for f, v in e.items()}
            assert max(e.values()) <= 1e-9, (s, e)
    assert gpu.t == pytest.approx(ref.t, rel=1e-9)
    print(json.dumps({"grid": 256, "steps": 50, "attempts": sum(attempts), "worst": worst,
                      "t": ref.t}))


def test_config0_adaptive_2000(built):
    """The small adaptive run (64^2, rel tol 1e-4, 2000 steps): the GPU's and
    the oracle's accept/reject sequences are compared step by step.  dt comes
    from the Merson error estimate, a difference of stage derivatives that
    cancels to O(dt^4) and amplifies rounding, so the step sizes of two
    correct implementations drift apart by more than the state's own rounding
    (attempt counts stay equal while dt differs in the last digits).  The
    oracle is therefore also run from inputs perturbed by 1e-15 (relative):
    up to the first step whose attempt count differs, each field must agree
    with the oracle within 1e-8 or 10x the oracle's own drift from the
    perturbed run, whichever is larger."""
    from oracle import oracle
    cfg, mesh, k, st, gpu, ref = _pair(64, seed=1, oracle_direct=True)
    rng = np.random.default_rng(0)
    st2 = {f: (np.asfortranarray(v * (1 + 1e-15 * rng.standard_normal(v.shape))) if f != "ph" else v)
           for f, v in st.items()}
    ref2 = oracle.OracleDischarge(cfg.replace(lapl_maxit=20000), mesh, st2, solver=oracle.SOLVER_DIRECT)
    diverged, self_diverged, rows = None, None, []
    for s in range(2002):
        gi, ri, r2 = gpu.step(), ref.step(), ref2.step()
        assert gi["lerr"] == 0 and ri["lerr"] == 0 and r2["lerr"] == 0, (s, gi, ri)
        if s >= 2 and gi["attempts"] != ri["attempts"] and diverged is None:
            diverged = s - 1
        if s >= 2 and r2["attempts"] != ri["attempts"] and self_diverged is None:
            self_diverged = s - 1
        if diverged is None and (s % 50 == 1 or s == 2001):
            rd = ref.download()
            e = field_errors(gpu.download(), rd, k["n_zero"])
            fl = field_errors(ref2.download(), rd, k["n_zero"])
            rows.append({"step": s - 1, "err": e, "oracle_self": fl,
                         "dt_rel": abs(gpu.dt - ref.dt) / ref.dt})
            for f in e:
                assert e[f] <= max(1e-8, 10 * fl[f]), (s - 1, f, e, fl)
    print(json.dumps({"grid": 64, "steps": 2000, "first_divergent_step": diverged,
                      "oracle_self_first_divergent_step": self_diverged,
                      "t_gpu": gpu.t, "t_oracle": ref.t, "checkpoints": rows}))
    assert diverged is None or diverged >= 200, diverged
