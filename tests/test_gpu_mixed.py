"""Mixed-precision path (FS_PREC_MIXED) against the FP64 oracle and the FP64
GPU path on identical seeded inputs (needs a GB300).

Bars: densities within 1e-5 relative to the FP64 result (L-infinity over the
interior with the density floor as absolute guard, and L2), phi within 1e-5
relative to max|phi|; every Poisson solve converged to the same relative
residual as the FP64 solver (lapl_rtol, here 1e-8), with the residual formed
in FP64.

Both runs take the same steps.  With the adaptive controller the FP32
right-hand side moves the Merson error estimate (a difference of stage
derivatives that cancels to O(dt^4)) by ~1e-4 relative, so two adaptive runs
drift apart in dt and, after tens of steps, sit at different times; that is a
different trajectory, not an arithmetic error.  The adaptive comparison
therefore replays the mixed run's accepted step sizes in an FP64 run with the
controller off.
"""
import numpy as np
import pytest

from tests._util import field_errors

pytestmark = pytest.mark.gpu

DENS_BAR = 1e-5


def _setup(n, seed=7, **kw):
    from fluidsim_gb300 import abi, api, config, grid
    cfg = config.glow(n, lapl_rtol=1e-8, **kw)
    mesh = cfg.mesh()
    k = api.constants(cfg)
    st = grid.blob_state(mesh, k, noise=0.01, seed=seed, vl=cfg.vl)
    return cfg, cfg.replace(precision=abi.FS_PREC_MIXED), mesh, k, st


def _l2(a, b):
    a = np.asarray(a)[1:-1, 1:-1]
    b = np.asarray(b)[1:-1, 1:-1]
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def _errors(g, r, k):
    e = field_errors(g, r, k["n_zero"])
    for f in ("ni", "ne", "nt"):
        e[f + "_l2"] = _l2(g[f], r[f])
    return e


def test_mixed_fixed_dt_vs_oracle(built):
    """20 fixed-dt steps on a 48x40 grid against the FP64 oracle."""
    from fluidsim_gb300 import api
    from oracle import oracle
    cfg, cfgm, mesh, k, st = _setup(48, ny=40, adaptive=0)
    cfg, cfgm = cfg.replace(dt0=cfg.dt0 / 4), cfgm.replace(dt0=cfg.dt0 / 4)
    gpu = api.Discharge(cfgm, mesh, st)
    ref = oracle.OracleDischarge(cfg, mesh, st, solver=oracle.SOLVER_DIRECT)
    for s in range(20):
        gi, ri = gpu.step(), ref.step()
        assert gi["lerr"] == 0 and ri["lerr"] == 0
        assert gi["relres"] <= cfg.lapl_rtol
    e = _errors(gpu.download(), ref.download(), k)
    assert max(e.values()) < DENS_BAR, e


@pytest.mark.parametrize("n,steps", [(128, 200), (256, 100)])
def test_mixed_fixed_dt_vs_fp64_gpu(built, n, steps):
    """Fixed-dt runs in both precisions through the C ABI; the FP64 GPU path
    stands for the oracle here (it matches the oracle to 1e-10)."""
    from fluidsim_gb300 import api
    cfg, cfgm, mesh, k, st = _setup(n, adaptive=0)
    cfg, cfgm = cfg.replace(dt0=cfg.dt0 / 4), cfgm.replace(dt0=cfg.dt0 / 4)
    a, b = api.Discharge(cfg, mesh, st), api.Discharge(cfgm, mesh, st)
    for s in range(steps):
        ga, gb = a.step(), b.step()
        assert ga["lerr"] == 0 and gb["lerr"] == 0, (s, ga, gb)
        assert gb["relres"] <= cfg.lapl_rtol
    e = _errors(b.download(), a.download(), k)
    assert max(e.values()) < DENS_BAR, e


def _replay(a, b, steps):
    """Step b (mixed, adaptive) and replay its step sizes in a (FP64, controller
    off).  The reference's loop runs lapl_solve with the dt the controller has
    already updated and advances t by it (main.F90:75-90), so a takes the
    attempt's dt in ptcl_step and b's updated dt in lapl_solve."""
    for s in range(steps):
        gb = b.step()
        assert gb["lerr"] == 0 and gb["relres"] <= b.cfg.lapl_rtol, (s, gb)
        if a.ts > 1:
            a.dt = b.stats()["dt_step"]   # the accepted attempt's dt
            a.ptcl_step()
        a.dt = b.dt
        ga = a.lapl_solve()
        assert ga["lerr"] == 0, (s, ga)
        a.accept()
    assert a.t == pytest.approx(b.t, rel=1e-14)


@pytest.mark.parametrize("n,steps", [(64, 150), (256, 60)])
def test_mixed_adaptive_replay(built, n, steps):
    from fluidsim_gb300 import api
    cfg, cfgm, mesh, k, st = _setup(n)
    a = api.Discharge(cfg.replace(adaptive=0), mesh, st)
    b = api.Discharge(cfgm, mesh, st)
    _replay(a, b, steps)
    e = _errors(b.download(), a.download(), k)
    assert max(e.values()) < DENS_BAR, e


def test_mixed_poisson_residual(built):
    """One mixed Poisson solve reaches the FP64 solver's relative residual in
    a comparable number of iterations, and its correction matches."""
    from fluidsim_gb300 import api
    cfg, cfgm, mesh, k, st = _setup(256)
    cfg = cfg.replace(lapl_rtol=1e-10)
    cfgm = cfgm.replace(lapl_rtol=1e-10)
    a, b = api.Discharge(cfg, mesh, st), api.Discharge(cfgm, mesh, st)
    ra, rb = a.lapl_solve(), b.lapl_solve()
    assert ra["lerr"] == 0 and rb["lerr"] == 0
    assert rb["relres"] <= 1e-10
    assert rb["iters"] <= ra["iters"] + 4, (ra, rb)
    pa, pb = a.download()["ph"], b.download()["ph"]
    assert np.max(np.abs(pa - pb)) <= 1e-6 * np.max(np.abs(pa))


def _sig_err(a, b):
    err = 0.0
    for key in ("sig_pl", "sig_mi", "sig_or"):
        scale = max(np.max(np.abs(b[key])), 1e-300)
        err = max(err, float(np.max(np.abs(a[key] - b[key])) / scale))
    return err


@pytest.mark.parametrize("cyl", [0, 1])
def test_mixed_dielectric_wall_vs_oracle(built, cyl):
    """The dielectric wall (type_y = 3 on the last row, surface charge by the
    Merson stages of sfc_lib.F90) in mixed precision: 20 fixed-dt steps on a
    40x32 grid against the FP64 oracle, a charged wall from the start.  Bars:
    1e-5 per field as above, 1e-5 for the three surface-charge arrays
    relative to their largest entry."""
    from fluidsim_gb300 import abi, api, config, grid
    from oracle import oracle
    cfg = config.glow(40, ny=32, lapl_rtol=1e-8).replace(cyl=cyl, rwall=True, adaptive=0)
    cfg = cfg.replace(dt0=cfg.dt0 / 4)
    mesh = cfg.mesh()
    k = api.constants(cfg)
    st = grid.blob_state(mesh, k, noise=0.01, seed=6, vl=cfg.vl)
    gpu = api.Discharge(cfg.replace(precision=abi.FS_PREC_MIXED), mesh, st)
    ref = oracle.OracleDischarge(cfg, mesh, st, solver=oracle.SOLVER_DIRECT)
    sig0 = 2e3 * np.sin(np.linspace(0.0, np.pi, cfg.nx + 2))
    for d in (gpu, ref):
        d.set_surface_charge(sig0, sig0, sig0)
    for s in range(20):
        gi, ri = gpu.step(), ref.step()
        assert gi["lerr"] == 0 and ri["lerr"] == 0, (s, gi, ri)
        assert gi["relres"] <= cfg.lapl_rtol
    e = _errors(gpu.download(), ref.download(), k)
    sg, sr = gpu.surface_charge(), ref.surface_charge()
    assert np.any(sr["sig_pl"][1:-1] != sig0[1:-1])
    e["sig"] = _sig_err(sg, sr)
    assert max(e.values()) < DENS_BAR, e


def test_mixed_dielectric_wall_vs_fp64_gpu(built):
    """The wall at 128x128 for 100 fixed-dt steps in both precisions."""
    from fluidsim_gb300 import api
    cfg, cfgm, mesh, k, st = _setup(128, adaptive=0, rwall=True)
    cfg, cfgm = cfg.replace(dt0=cfg.dt0 / 4), cfgm.replace(dt0=cfg.dt0 / 4)
    a, b = api.Discharge(cfg, mesh, st), api.Discharge(cfgm, mesh, st)
    sig0 = 2e3 * np.sin(np.linspace(0.0, np.pi, cfg.nx + 2))
    for d in (a, b):
        d.set_surface_charge(sig0, sig0, sig0)
    for s in range(100):
        ga, gb = a.step(), b.step()
        assert ga["lerr"] == 0 and gb["lerr"] == 0, (s, ga, gb)
    e = _errors(b.download(), a.download(), k)
    e["sig"] = _sig_err(b.surface_charge(), a.surface_charge())
    assert max(e.values()) < DENS_BAR, e


@pytest.mark.parametrize("rf,t0,res_scale", [(1, 0.25, 1e-3), (1, 0.6, 1.0), (2, 0.1, 1.0), (3, 0.3, 1.0)])
def test_mixed_sources_vs_oracle(built, rf, t0, res_scale):
    """The AC source through the RC circuit (rf = 1, one circuit kernel per
    stage) and the two pulse shapes (rf = 2, 3) in mixed precision, electrodes
    on part of the wall: 20 fixed-dt steps against the FP64 oracle.  Bars:
    1e-5 per field; the electrode voltages to 1e-5 relative, and for the RC
    circuit its change over the run to 1e-4 relative."""
    from fluidsim_gb300 import abi, api, config, grid
    from oracle import oracle
    cfg = config.glow(40, ny=32, rf=rf, ew=2.0, gap=10.0, lapl_rtol=1e-8, adaptive=0)
    cfg = cfg.replace(res=cfg.res * res_scale, dt0=cfg.dt0 / 4)
    mesh = cfg.mesh()
    k = api.constants(cfg)
    st = grid.blob_state(mesh, k, noise=0.01, seed=8, vl=cfg.vl)
    gpu = api.Discharge(cfg.replace(precision=abi.FS_PREC_MIXED), mesh, st)
    ref = oracle.OracleDischarge(cfg, mesh, st, solver=oracle.SOLVER_DIRECT)
    for d in (gpu, ref):
        d.set_time(t0, cfg.dt0)
    v_start = ref.circuit()["vd_pl"]
    for s in range(20):
        gi, ri = gpu.step(), ref.step()
        assert gi["lerr"] == 0 and ri["lerr"] == 0, (s, gi, ri)
        assert gi["relres"] <= cfg.lapl_rtol
    e = _errors(gpu.download(), ref.download(), k)
    assert max(e.values()) < DENS_BAR, e
    cg, cr = gpu.circuit(), ref.circuit()
    for key in ("vd_pl", "vd_mi", "vd_or", "vsrc"):
        assert abs(cg[key] - cr[key]) <= 1e-5 * abs(cr[key]) + 1e-300, (key, cg, cr)
    if rf == 1:
        moved = cr["vd_pl"] - v_start
        assert moved != 0.0
        assert abs((cg["vd_pl"] - v_start) - moved) <= 1e-4 * abs(moved), (cg, cr, v_start)
