"""Failure detection without a GPU fault (needs a GB300): every failure is
injected on the host -- a planted NaN or negative density in an uploaded
state, a Krylov iteration cap too small to converge, a minimum dt above the
step size, a first step too large for the error controller -- and the library
must report it as the reference does (get_Te's stop ptcl_props.F90:171-177,
KSP divergence -> lerr = 1 lapl_lib.F90:104-109, the minimum-dt stop
ptcl_lib.F90:68-72, the reject-and-retry loop ptcl_lib.F90:74-94) and stay
usable afterwards.  Also the odd and tiny grids against the oracle."""
import numpy as np
import pytest

from tests._util import field_errors

pytestmark = pytest.mark.gpu


def _setup(n=24, ny=20, **kw):
    from fluidsim_gb300 import api, config, grid
    cfg = config.glow(n, ny=ny, lapl_rtol=1e-12, **kw)
    mesh = cfg.mesh()
    k = api.constants(cfg)
    st = grid.blob_state(mesh, k, noise=0.01, seed=11, vl=cfg.vl)
    return cfg, mesh, k, st


@pytest.mark.parametrize("precision", [0, 1])
@pytest.mark.parametrize("bad", ["nan", "negative"])
def test_planted_bad_density_is_reported(built, precision, bad):
    from fluidsim_gb300 import abi, api
    cfg, mesh, k, st = _setup(precision=precision)
    d = api.Discharge(cfg, mesh, st)
    for _ in range(3):
        d.step()
    good = d.download(nlev=3)
    t, dt, ts = d.t, d.dt, d.ts
    broken = {f: np.array(v, copy=True, order="F") for f, v in good.items() if v is not None}
    broken["ne"][9, 7, 1] = np.nan if bad == "nan" else -1.0   # level 2: the stage state
    d.upload(broken)
    with pytest.raises(api.FluidsimError) as ei:
        d.ptcl_step()
    assert ei.value.code in (abi.FS_ERR_NEG_DENSITY, abi.FS_ERR_NAN), ei.value
    # the context stays usable: the good state goes back and stepping resumes
    d.upload(good)
    d.set_time(t, dt)
    d.ts = ts
    for _ in range(3):
        assert d.step()["lerr"] == 0


@pytest.mark.parametrize("precision", [0, 1])
def test_krylov_cap_gives_lerr_and_keeps_phi(built, precision):
    """A solve that cannot reach lapl_rtol in lapl_maxit iterations reports
    lerr = 1 and leaves phi as it was; fs_run then rejects the step: dt
    halves and the levels are restored (main.F90:102-121)."""
    from fluidsim_gb300 import api
    cfg, mesh, k, st = _setup(64, 64, precision=precision, lapl_maxit=2)
    d = api.Discharge(cfg, mesh, st)
    ph0 = d.download()["ph"]
    r = d.lapl_solve()
    assert r["lerr"] == 1 and r["iters"] <= 2, r
    assert np.array_equal(d.download()["ph"], ph0)
    dt = d.dt
    stats = d.run(1)
    assert stats["lapl_rejects"] == 1 and stats["steps"] == 0
    assert d.dt == dt / 2


def test_min_dt_stop(built):
    from fluidsim_gb300 import abi, api
    cfg, mesh, k, st = _setup()
    cfg = cfg.replace(dt_min=10 * cfg.dt0)
    d = api.Discharge(cfg, mesh, st)
    for _ in range(2):
        d.step()
    with pytest.raises(api.FluidsimError) as ei:
        d.ptcl_step()
    assert ei.value.code == abi.FS_ERR_MIN_DT


def test_rk_reject_and_retry_matches_oracle(built):
    """A first step far above what the error controller accepts: the attempt
    is rejected and retried with the smaller dt, in the same way as the
    oracle (same attempts, same dt, fields to 1e-10)."""
    from fluidsim_gb300 import api
    from oracle import oracle
    cfg, mesh, k, st = _setup(32, 24)
    cfg = cfg.replace(dt0=cfg.dt0 * 20)
    gpu = api.Discharge(cfg, mesh, st)
    ref = oracle.OracleDischarge(cfg, mesh, st, solver=oracle.SOLVER_DIRECT)
    saw_retry = False
    for s in range(6):
        gi, ri = gpu.step(), ref.step()
        assert gi["lerr"] == ri["lerr"] == 0
        if s >= 2:
            assert gi["attempts"] == ri["attempts"], (s, gi, ri)
            saw_retry |= gi["attempts"] > 1
            assert abs(gi["dt"] - ri["dt"]) <= 1e-9 * abs(ri["dt"])
    assert saw_retry
    e = field_errors(gpu.download(), ref.download(), k["n_zero"])
    assert max(e.values()) < 1e-10, e


@pytest.mark.parametrize("nx,ny", [(3, 2), (3, 3), (5, 7), (7, 5), (33, 17)])
@pytest.mark.parametrize("precision", [0, 1])
def test_tiny_and_odd_grids_vs_oracle(built, nx, ny, precision):
    from fluidsim_gb300 import api
    from oracle import oracle
    cfg, mesh, k, st = _setup(nx, ny, precision=precision, adaptive=0)
    gpu = api.Discharge(cfg, mesh, st)
    ref = oracle.OracleDischarge(cfg.replace(precision=0), mesh, st, solver=oracle.SOLVER_DIRECT)
    for _ in range(5):
        gi, ri = gpu.step(), ref.step()
        assert gi["lerr"] == 0 and ri["lerr"] == 0, (gi, ri)
    e = field_errors(gpu.download(), ref.download(), k["n_zero"])
    assert max(e.values()) < (1e-10 if precision == 0 else 1e-5), e
