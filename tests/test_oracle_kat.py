"""Known-answer tests of the CPU oracle, derived from the mathematics (the
reference has no tests or golden data of its own):
  * get_Flux (ptcl_props.F90:142-165): diffusion limit, drift limit,
    mirror symmetry, the exp(-100) clamp;
  * dFdPh (lapl_lib.F90:611-636) is the derivative of the SG flux in v;
  * RK-Merson (ptcl_props.F90:71-139) is 4th order on the source-only ODE
    of a uniform plasma between zero-flux walls, and leaves it uniform;
  * the Poisson system (lapl_lib.F90:123-609) reproduces a linear potential
    exactly, converges at 2nd order on a manufactured solution, and is
    symmetric after scaling each row by its control volume;
  * the anode and cathode currents of circ_step (circ_lib.F90:87-151) come
    together as a discharge approaches steady state (current continuity).
"""
import math

import numpy as np
import pytest

from fluidsim_gb300 import abi, api, config, grid
from oracle import oracle


def flux(E, dh, q, mu, D, nl, nr):
    return oracle.get_flux(E, dh, q, mu, D, nl, nr)


def test_flux_diffusion_limit():
    # |qE| below 1e-12: pure diffusion D (nl - nr)/dh, and continuity just above it
    assert flux(0.0, 2.0, 1, 3.0, 5.0, 7.0, 4.0) == pytest.approx(5.0 * 3.0 / 2.0, rel=1e-15)
    f_small = flux(1e-9, 2.0, -1, 3.0, 5.0, 7.0, 4.0)
    assert f_small == pytest.approx(7.5, rel=1e-8)


def test_flux_drift_limit():
    # D -> 0 (|a| >> 1): upwind drift v * n_upwind
    v = 2.0 * 10.0
    assert flux(10.0, 1.0, 1, 2.0, 1e-3, 3.0, 5.0) == pytest.approx(v * 3.0, rel=1e-12)
    assert flux(-10.0, 1.0, 1, 2.0, 1e-3, 3.0, 5.0) == pytest.approx(-v * 5.0, rel=1e-12)


@pytest.mark.parametrize("E", [3.7, -0.2, 1e-3, 55.0, -400.0])
@pytest.mark.parametrize("q", [1, -1])
def test_flux_mirror(E, q):
    a = flux(E, 0.7, q, 1.3, 0.9, 2.0, 5.0)
    b = flux(-E, 0.7, q, 1.3, 0.9, 5.0, 2.0)
    assert a == pytest.approx(-b, rel=1e-13, abs=1e-300)
    assert a == pytest.approx(flux(-E, 0.7, -q, 1.3, 0.9, 2.0, 5.0), rel=1e-15)


def test_flux_clamp():
    # arg = 400: exp(max(-arg, -100)) = exp(-100) in numerator and denominator
    E, dh, mu, D, nl, nr = 400.0, 1.0, 1.0, 1.0, 1.0, 1e60
    e = math.exp(-100.0)
    want = 400.0 * (nl - nr * e) / (1.0 - e)
    assert flux(E, dh, 1, mu, D, nl, nr) == pytest.approx(want, rel=1e-14)


@pytest.mark.parametrize("E", [0.3, -2.0, 17.0, -60.0, 1e-4, -3e-3, 4.7e-3])
@pytest.mark.parametrize("q", [1, -1])
def test_dfdph_is_flux_derivative(E, q):
    mu, D, dx, n1, n2 = 1.7, 0.8, 0.6, 3.0, 1.2
    h = 1e-6 * max(1.0, abs(E))
    num = (flux(E + h, dx, q, mu, D, n1, n2) - flux(E - h, dx, q, mu, D, n1, n2)) / (2 * h)
    # d flux / dE = q mu d flux / dv
    got = q * mu * oracle.dfdph(E, E, q, mu, D, dx, n1, n2)
    assert got == pytest.approx(num, rel=1e-6)


def test_dfdph_continuous_across_series_branch():
    # |a| = 0.05 separates the series from the closed form; both sides agree
    mu, D, dx, n1, n2 = 2.0, 1.0, 0.5, 3.0, 1.0
    E0 = 0.05 * D / (mu * dx)
    lo = oracle.dfdph(E0 * (1 - 1e-13), E0 * (1 - 1e-13), 1, mu, D, dx, n1, n2)
    hi = oracle.dfdph(E0 * (1 + 1e-13), E0 * (1 + 1e-13), 1, mu, D, dx, n1, n2)
    assert lo == pytest.approx(hi, rel=1e-12)
    # and the a -> 0 limit is the mean density
    tiny = oracle.dfdph(1e-11, 1e-11, 1, mu, D, dx, n1, n2)
    assert tiny == pytest.approx(0.5 * (n1 + n2), rel=1e-10)


def _vacuum_cfg(n=6, **kw):
    # walls are Neumann (type -1/+1) on all four sides: ew < 0 and gap beyond the domain
    return config.glow(n, ny=n - 1, ew=-1.0, gap=1e9, vl=0.0, mesh_law="uniform", adaptive=0,
                       coef_mode=abi.FS_COEF_FITS, **kw)


def _uniform_state(cfg, mesh, n0, eps_ev):
    shp = (cfg.nx + 2, cfg.ny + 2)
    ne = np.full(shp, n0, order="F")
    return dict(ni=ne.copy(order="F"), ne=ne, nt=np.asfortranarray(ne * eps_ev / config.PH0),
                ph=np.zeros(shp, order="F"))


def _ode_rhs(o, k, y):
    """Source terms of ptclEqn (ptcl_lib.F90:482-523) for a uniform plasma, E = 0."""
    ni, ne, nt = y
    T = nt / ne
    c = [o.coef(w, T) for w in range(6)]
    k_ir, k_ex, nu, beta = c[2], c[3], c[4], c[5]
    sie = k_ir * k["ninf"] * ne - beta * ni * ne
    st2 = -(ne * nu * k["me"] / k["mi"] * (T / 1.5 - k["tg"] * k["kb"] / k["e"] / k["ph0"]))
    st3 = -(k["h_ir"] * k_ir * k["ninf"] * ne) - k["h_ex"] * k_ex * k["ninf"] * ne
    return np.array([sie, sie, st2 + st3])


def _ode_exact(o, k, y0, t):
    from scipy.integrate import solve_ivp
    sol = solve_ivp(lambda _t, y: _ode_rhs(o, k, y), (0.0, t), y0, method="DOP853",
                    rtol=1e-13, atol=1e-16)
    return sol.y[:, -1]


def test_merson_order_and_uniformity(built):
    cfg = _vacuum_cfg()
    mesh = cfg.mesh()
    k = api.constants(cfg, oracle.load(), "or_")
    n0, eps = 100.0, 4.0
    y0 = np.array([n0, n0, n0 * eps / config.PH0])
    errs = []
    for dt in (0.16, 0.08, 0.04):
        o = oracle.OracleDischarge(cfg, mesh, _uniform_state(cfg, mesh, n0, eps))
        o.dt = dt
        o.ptcl_step()
        d = o.download()
        inner = {f: d[f][1:-1, 1:-1] for f in ("ni", "ne", "nt")}
        for f, a in inner.items():
            assert np.ptp(a) <= 1e-14 * abs(a).max(), f   # stays uniform
        got = np.array([inner["ni"][0, 0], inner["ne"][0, 0], inner["nt"][0, 0]])
        exact = _ode_exact(o, k, y0, dt)
        errs.append(abs(got[2] - exact[2]) / abs(exact[2]))   # the energy density moves most
        o.close()
    # local error of a 4th-order step scales as dt^5
    assert min(errs) > 1e-13, errs
    assert errs[0] / errs[1] > 20 and errs[1] / errs[2] > 20, errs


def _poisson_case(n, law, rho_fn, ghost=0.0):
    cfg = config.glow(n, ny=4, mesh_law=law, vl=0.0, adaptive=0)
    mesh = cfg.mesh()
    shp = (n + 2, 6)
    X = np.repeat(mesh.x[:, None], 6, axis=1)
    n0 = 1e3
    ne = np.full(shp, n0)
    ni = n0 + rho_fn(X)
    ph = np.zeros(shp)
    ph[0, :] = ghost
    ph[-1, :] = -ghost
    st = dict(ni=np.asfortranarray(ni), ne=np.asfortranarray(ne),
              nt=np.asfortranarray(ne / config.PH0), ph=np.asfortranarray(ph))
    o = oracle.OracleDischarge(cfg, mesh, st, solver=oracle.SOLVER_DIRECT)
    o.dt = 0.0
    r = o.lapl_solve()
    assert r["lerr"] == 0
    return mesh, o.download()["ph"]


@pytest.mark.parametrize("law", ["uniform", "geometric"])
def test_poisson_linear_potential_exact(built, law):
    V = 1000.0
    mesh, ph = _poisson_case(20, law, lambda X: 0.0 * X, ghost=V / 2)
    L = mesh.x[-1]
    want = V / 2 - V * mesh.x / L
    assert np.allclose(ph[1:-1, 1:-1], want[1:-1, None], rtol=0, atol=1e-11 * V)


def test_poisson_second_order(built):
    errs = []
    for n in (16, 32, 64):
        L = config.glow(n).l
        k2 = (math.pi / L) ** 2
        mesh, ph = _poisson_case(n, "uniform", lambda X: 1e2 * k2 * np.sin(math.pi * X / L))
        exact = 1e2 * np.sin(math.pi * mesh.x / L)
        errs.append(np.max(np.abs(ph[1:-1, 2] - exact[1:-1])))
    assert 3.5 < errs[0] / errs[1] < 4.5 and 3.5 < errs[1] / errs[2] < 4.5, errs


def test_poisson_rows_symmetric_after_volume_scaling(built):
    cfg = config.glow(20, ny=12)
    mesh = cfg.mesh()
    k = api.constants(cfg, oracle.load(), "or_")
    st = grid.blob_state(mesh, k, noise=0.01, seed=2)
    st["ph"] = np.asfortranarray(np.linspace(-7e5, 7e5, 22)[:, None] * np.ones((1, 14)))
    o = oracle.OracleDischarge(cfg, mesh, st)
    b, a5 = o.assemble(1e-6)
    nx, ny = cfg.nx, cfg.ny
    D = (mesh.dlx[:, None] * mesh.dly[None, :]).ravel(order="F")
    A = a5 * D[:, None]
    for j in range(ny):
        for i in range(nx):
            q = i + j * nx
            if i + 1 < nx:
                assert A[q, 1] == pytest.approx(A[q + 1, 0], rel=1e-14)
            if j + 1 < ny:
                assert A[q, 3] == pytest.approx(A[q + nx, 2], rel=1e-14)
    # diagonally dominant M-matrix rows: -A_c >= sum of off-diagonals
    assert np.all(-A[:, 4] >= A[:, :4].sum(axis=1) * (1 - 1e-12))


@pytest.mark.parametrize("a", [3e-17, 1e-14, 1e-9, 1e-4, 0.0099, 0.0101, 0.3, 7.0])
@pytest.mark.parametrize("q", [1, -1])
def test_flux_matches_high_precision(a, q):
    """get_Flux against a 50-digit evaluation of the same function: the small
    Peclet branch (|a| < 1e-2) and the closed form both hold to ~1e-14."""
    mp = pytest.importorskip("mpmath")
    mp.mp.dps = 50
    mu, D, dh, nl, nr = 1e-3, 1e3, 0.5, 3.0, 2.0   # |E| stays above the 1e-12 cut
    E = q * a * D / (mu * dh)          # so that arg = q*mu*E*dh/D = a
    assert abs(E) > 1e-12
    v = mp.mpf(q) * mu * mp.mpf(E)
    A = v * dh / D
    exact = v * (nl - nr * mp.e ** (-A)) / (1 - mp.e ** (-A))
    got = flux(E, dh, q, mu, D, nl, nr)
    assert abs(got - float(exact)) <= 2e-14 * float(abs(exact)), (got, exact)


@pytest.mark.parametrize("a", [1e-12, 1e-7, 0.049, 0.051, 2.0])
def test_dfdph_matches_high_precision(a):
    mp = pytest.importorskip("mpmath")
    mp.mp.dps = 50
    mu, D, dx, n1, n2 = 1.1, 0.9, 0.5, 4.0, 1.5
    E = a * D / (mu * dx)

    def F(vv):
        A = vv * dx / D
        return vv * (n1 - n2 * mp.e ** (-A)) / (1 - mp.e ** (-A))
    exact = mp.diff(F, mp.mpf(mu) * mp.mpf(E))
    got = oracle.dfdph(E, E, 1, mu, D, dx, n1, n2)
    assert abs(got - float(exact)) <= 1e-12 * float(abs(exact)), (got, exact)


def test_current_continuity_approaching_steady_state(built):
    """Ida = Idc at steady state (current continuity): a 1D-like 400 V
    discharge (32 x 2 nodes, electrodes on every row with current weight)
    grows from the seed blob; the anode and cathode conduction currents,
    far apart while the space charge builds up, agree to 1 % after ~2.7 us
    (60,000 adaptive steps) and the difference keeps falling."""
    cfg = config.glow(32, ny=2, ew=10.0, gap=20.0, lapl_rtol=1e-10, vl=-400.0 / config.PH0)
    mesh = cfg.mesh()
    k = api.constants(cfg, oracle.load(), "or_")
    st = grid.blob_state(mesh, k, noise=0.0, seed=1, vl=cfg.vl)
    o = oracle.OracleDischarge(cfg, mesh, st)
    rel = []
    for chunk in range(6):
        o.run(10000)
        s = o.stats()
        rel.append(abs(s["ida"] - s["idc"]) / abs(s["idc"]))
    assert rel[0] > 0.5, rel            # early: space charge building up
    assert rel[-1] < 1e-2, rel          # late: continuity
    assert rel[-1] < rel[0] / 50, rel
