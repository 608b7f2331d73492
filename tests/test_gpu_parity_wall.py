"""Cylindrical geometry (cyl, r-weighted divergence and Poisson rows) and the
dielectric wall (type_y = 3 on the last row with the surface-charge Merson
stages of sfc_lib.F90) on the GPU against the CPU oracle on identical seeded
inputs (needs a GB300).  Bars: 1e-10 per field as for the Cartesian glow
(relative, density floor as absolute guard; phi relative to max|phi|), and
1e-10 for the three surface-charge arrays relative to their largest entry."""
import numpy as np
import pytest

from tests._util import field_errors, rel_linf

pytestmark = pytest.mark.gpu

CASES = [  # cyl, rwall, nspecies, coefficient fits, adaptive
    (1, False, 3, False, 1),
    (0, True, 3, False, 1),
    (1, True, 3, False, 0),
    (1, True, 4, True, 1),
]


def _cfg(cyl, rwall, ns, fits, adaptive):
    from fluidsim_gb300 import config
    if fits:
        cfg = config.reference_defaults(40, 32)
    else:
        cfg = config.glow(40, ny=32)
    return cfg.replace(cyl=cyl, rwall=rwall, nspecies=ns, adaptive=adaptive, lapl_rtol=1e-14)


def _sig_err(a, b):
    err = 0.0
    for key in ("sig_pl", "sig_mi", "sig_or"):
        scale = max(np.max(np.abs(b[key])), 1e-300)
        err = max(err, float(np.max(np.abs(a[key] - b[key])) / scale))
    return err


@pytest.mark.parametrize("cyl,rwall,ns,fits,adaptive", CASES)
def test_wall_and_cylinder_vs_oracle(built, cyl, rwall, ns, fits, adaptive):
    from fluidsim_gb300 import api, grid
    from oracle import oracle
    cfg = _cfg(cyl, rwall, ns, fits, adaptive)
    mesh = cfg.mesh()
    k = api.constants(cfg)
    st = grid.blob_state(mesh, k, noise=0.01, seed=6, vl=cfg.vl)
    if ns == 4:
        st["nm"] = np.asfortranarray(0.1 * st["ni"])
    gpu = api.Discharge(cfg, mesh, st)
    ref = oracle.OracleDischarge(cfg, mesh, st, solver=oracle.SOLVER_DIRECT)
    if rwall:
        # a charged wall from the start, so that its field drives the wall fluxes
        sig0 = 2e3 * np.sin(np.linspace(0.0, np.pi, cfg.nx + 2))
        for d in (gpu, ref):
            d.set_surface_charge(sig0, sig0, sig0)
    for s in range(8):
        gi, ri = gpu.step(), ref.step()
        assert gi["lerr"] == 0 and ri["lerr"] == 0, (s, gi, ri)
        if s >= 2 and adaptive:
            assert gi["attempts"] == ri["attempts"], (s, gi, ri)
            assert abs(gi["dt"] - ri["dt"]) <= 1e-6 * abs(ri["dt"]), (s, gi, ri)
    g, r = gpu.download(), ref.download()
    e = field_errors(g, r, k["n_zero"])
    if ns == 4:
        e["nm"] = rel_linf(g["nm"], r["nm"], k["n_zero"])
    if rwall:
        sg, sr = gpu.surface_charge(), ref.surface_charge()
        assert np.any(sr["sig_pl"][1:-1] != sr["sig_or"][1:-1])
        e["sig"] = _sig_err(sg, sr)
    assert max(e.values()) < 1e-10, e


def test_wall_reject_restores_charge(built):
    """A Poisson rejection (main.F90:103-121) sets sig_pl = sig_mi = sig_or on
    the device as in the oracle."""
    from fluidsim_gb300 import api, grid
    cfg = _cfg(0, True, 3, False, 0)
    mesh = cfg.mesh()
    k = api.constants(cfg)
    st = grid.blob_state(mesh, k, noise=0.01, seed=6, vl=cfg.vl)
    d = api.Discharge(cfg, mesh, st)
    rng = np.random.default_rng(2)
    pl, mi, orr = (rng.standard_normal(cfg.nx + 2) for _ in range(3))
    d.set_surface_charge(pl, mi, orr)
    d.accept()
    s = d.surface_charge()
    assert np.array_equal(s["sig_or"], mi) and np.array_equal(s["sig_mi"], pl) and np.array_equal(s["sig_pl"], pl)
    d.set_surface_charge(pl, mi, orr)
    d.reject()
    s = d.surface_charge()
    assert np.array_equal(s["sig_pl"], orr) and np.array_equal(s["sig_mi"], orr) and np.array_equal(s["sig_or"], orr)

