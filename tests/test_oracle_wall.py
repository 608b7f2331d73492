"""The oracle's dielectric wall (the reference's rwall: type_y = 3 on the
last row, sfc_lib.F90) on the CPU: mesh types, the surface-charge module
arrays through the accept / reject rotations of main.F90:83-121 and the
restart of ptcl_step (ptcl_lib.F90:83-93), and the wall field in the
Poisson system (lapl_lib.F90:72-76,263-265,548-600)."""
import numpy as np
import pytest

from fluidsim_gb300 import api, config, grid
from oracle import oracle


def _case(n=12, ny=10, **kw):
    cfg = config.glow(n, ny=ny, rwall=True, lapl_rtol=1e-14, **kw)
    mesh = cfg.mesh()
    k = api.constants(cfg, oracle.load(), "or_")
    st = grid.blob_state(mesh, k, noise=0.01, seed=4, vl=cfg.vl)
    return cfg, mesh, k, st


def test_mesh_marks_last_row():
    cfg = config.glow(8, ny=6, rwall=True)
    ty = cfg.mesh().type_y
    assert np.all(ty[:, -1] == 3) and np.all(ty[:, 0] == -1) and np.all(ty[:, 1:-1] == 0)
    assert np.all(config.glow(8, ny=6).mesh().type_y[:, -1] == 1)


def test_charge_starts_at_zero_and_charges_up(built):
    cfg, mesh, k, st = _case(adaptive=0)
    o = oracle.OracleDischarge(cfg, mesh, st)
    s = o.surface_charge()
    assert all(np.all(v == 0) for v in s.values())
    for _ in range(4):
        assert o.step()["lerr"] == 0
    s = o.surface_charge()
    wall = s["sig_pl"][1:-1]
    assert np.all(np.isfinite(wall)) and np.any(wall != 0)
    # ghost entries (no east/west neighbour on one block) stay untouched
    assert s["sig_pl"][0] == 0 and s["sig_pl"][-1] == 0


def test_accept_and_reject_rotations(built):
    cfg, mesh, k, st = _case(adaptive=0)
    o = oracle.OracleDischarge(cfg, mesh, st)
    rng = np.random.default_rng(1)
    pl, mi, orr = (rng.standard_normal(cfg.nx + 2) for _ in range(3))
    o.set_surface_charge(pl, mi, orr)
    o.accept()                       # sig_or <- sig_mi, sig_mi <- sig_pl
    s = o.surface_charge()
    assert np.array_equal(s["sig_or"], mi) and np.array_equal(s["sig_mi"], pl)
    assert np.array_equal(s["sig_pl"], pl)
    o.set_surface_charge(pl, mi, orr)
    o.reject()                       # sig_pl = sig_mi = sig_or
    s = o.surface_charge()
    assert np.array_equal(s["sig_pl"], orr) and np.array_equal(s["sig_mi"], orr)


def test_stage_combination_of_one_attempt(built):
    """After a fixed-dt attempt sig_or is untouched, sig_mi holds the stage-4
    value and sig_pl the stage-5 one; a second attempt from the same start
    reproduces them (the state is restored by the caller here)."""
    cfg, mesh, k, st = _case(adaptive=0)
    o = oracle.OracleDischarge(cfg, mesh, st)
    o.ts = 2
    sig0 = np.linspace(-50.0, 50.0, cfg.nx + 2)
    o.set_surface_charge(sig0, sig0, sig0)
    st0 = o.download(nlev=3)
    o.ptcl_step()
    s1 = o.surface_charge()
    assert np.array_equal(s1["sig_or"], sig0)
    assert np.any(s1["sig_pl"][1:-1] != sig0[1:-1]) and np.any(s1["sig_mi"][1:-1] != s1["sig_pl"][1:-1])
    p = oracle.OracleDischarge(cfg, mesh, None)
    p.upload(st0)
    p.set_time(o.t, cfg.dt0)
    p.set_surface_charge(sig0, sig0, sig0)
    p.ptcl_step()
    s2 = p.surface_charge()
    for key in s1:
        assert np.array_equal(s1[key], s2[key]), key


def test_wall_field_enters_poisson_rows(built):
    """The wall rows' b moves by the wall field change over dly; the
    matrix has no north column on the wall and an interior-form diagonal."""
    cfg, mesh, k, st = _case(adaptive=0)
    o = oracle.OracleDischarge(cfg, mesh, st)
    sig = np.zeros(cfg.nx + 2)
    sig[1:-1] = 3.0
    o.set_surface_charge(sig, None, None)
    b1, a1 = o.assemble(0.0)
    o.set_surface_charge(np.zeros(cfg.nx + 2), None, None)
    b2, a2 = o.assemble(0.0)
    nx, ny = cfg.nx, cfg.ny
    top = slice((ny - 1) * nx, ny * nx)
    # dt = 0: b = dfdx + dfdy + ni - ne; dfdy = -(Ey(2) - Ey(1))/dly with Ey(2) = -sig
    assert np.allclose(b1[top] - b2[top], 3.0 / mesh.dly[ny - 1], rtol=1e-12, atol=0)
    assert np.array_equal(b1[:(ny - 1) * nx], b2[:(ny - 1) * nx])
    assert np.all(a1[top, 3] == 0)
    want = -1.0 / mesh.dly[ny - 1] * (1.0 / mesh.dy[ny] + 1.0 / mesh.dy[ny - 1])
    inner = a2[top][1:-1]
    x_part = -(1.0 / mesh.dlx[1:-1]) * (1.0 / mesh.dx[2:-1] + 1.0 / mesh.dx[1:-2])
    assert np.allclose(inner[:, 4], x_part + want, rtol=1e-13, atol=0)
