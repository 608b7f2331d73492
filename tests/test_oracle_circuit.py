"""The oracle's external circuit on the CPU (circ_lib.F90:19-223): the source
waveforms of rf = 1, 2, 3 (:26-50), the RC circuit of the AC source
(:156-174) as a 4th-order Merson integration of dVd/dt = (Vsrc - Vd)/(R C)
when no electrode current flows, Vd = Vsrc for the other sources (:176-177),
and the ghost potentials +-Vd/2 it writes (:178-198)."""
import math

import numpy as np
import pytest

from fluidsim_gb300 import api, config, grid
from oracle import oracle


def _source(rf, V, t):
    pi = 4.0 * math.atan(1.0)
    if rf == 1:
        return V * math.sin(pi * t)
    if rf == 2:
        return V * math.sin(4 * pi * t) ** 3 if t < 0.25 else 0.0
    if rf == 3:
        if t < 0.23:
            return V * math.sin(4 * pi * t) ** 2
        if t < 0.335:
            return V * (math.sin(3.81 * pi * (t + 0.0585)) * 0.719 + 0.281)
        if t < 0.82:
            return V * (math.sin(3.81 * pi * (t + 0.12) / 3.5) ** 3 * (-0.438))
        return 0.0
    return V


def _disch(rf, t, **kw):
    cfg = config.glow(16, ny=12, rf=rf, adaptive=0, lapl_rtol=1e-14, **kw)
    mesh = cfg.mesh()
    k = api.constants(cfg, oracle.load(), "or_")
    st = grid.blob_state(mesh, k, noise=0.01, seed=3, vl=cfg.vl)
    o = oracle.OracleDischarge(cfg, mesh, st)
    o.set_time(t, cfg.dt0)
    return cfg, mesh, k, o


@pytest.mark.parametrize("rf,t", [(2, 0.1), (2, 0.3), (3, 0.1), (3, 0.3), (3, 0.5), (3, 0.9)])
def test_pulse_sources_set_vd(built, rf, t):
    cfg, mesh, k, o = _disch(rf, t)
    o.ptcl_step()
    c = o.circuit()
    want = _source(rf, cfg.vl, t)
    assert c["vsrc"] == pytest.approx(want, rel=1e-14, abs=1e-300)
    assert c["vd_pl"] == c["vsrc"] and c["vd_mi"] == c["vsrc"]
    ph = o.download()["ph"]
    assert np.all(ph[0, 1:-1] == c["vd_pl"] / 2.0) and np.all(ph[-1, 1:-1] == c["vd_pl"] / -2.0)


def _merson_linear(v0, s, lam, dt):
    """The five Merson stages of circ_step on dV/dt = lam (V - s)."""
    kv = [0.0] * 6
    vmi = v0
    for stage in range(1, 6):
        kv[stage] = lam * (vmi - s)
        if stage == 1: vmi = v0 + dt * kv[1] / 3.0
        elif stage == 2: vmi = v0 + dt * (kv[1] + kv[2]) / 6.0
        elif stage == 3: vmi = v0 + dt * (kv[1] + kv[3] * 3.0) / 8.0
        elif stage == 4: vmi = v0 + dt * (kv[1] - kv[3] * 3.0 + kv[4] * 4.0) / 2.0
        else: vpl = v0 + dt * (kv[1] + kv[4] * 4.0 + kv[5]) / 6.0
    return vpl, vmi


def test_ac_rc_circuit_is_merson_on_the_rc_equation(built):
    """With electrodes over the whole wall the current rows carry no weight
    (dr = 0 where r < ew, circ_lib.F90:97,130), so Idc = 0 and the electrode
    voltage obeys dVd/dt = (Vsrc - Vd)/(Res Cap) with Vsrc frozen at the step's
    time.  One attempt equals the Merson stages on that equation, and its
    error against the exact exponential falls as dt^5."""
    errs = []
    for scale in (1.0, 0.5, 0.25):
        cfg, mesh, k, o = _disch(1, 0.25)
        rc = cfg.res * k["cap"]
        dt = 0.4 * rc * scale
        res = cfg.res
        o.dt = dt
        v0 = 0.3 * cfg.vl
        o.set_circuit(v0, v0, v0)
        o.ptcl_step()
        c = o.circuit()
        assert o.stats()["idc"] == 0.0
        s = _source(1, cfg.vl, 0.25)
        vpl, vmi = _merson_linear(v0, s, -1.0 / (res * k["cap"]), dt)
        assert c["vd_pl"] == pytest.approx(vpl, rel=1e-14)
        assert c["vd_mi"] == pytest.approx(vmi, rel=1e-14)
        exact = s + (v0 - s) * math.exp(-dt / rc)
        errs.append(abs(c["vd_pl"] - exact) / abs(v0 - s))
        ph = o.download()["ph"]
        assert np.all(ph[0, 1:-1] == c["vd_pl"] / 2.0)
    assert errs[0] / errs[1] > 24 and errs[1] / errs[2] > 24, errs


def test_circuit_rotation(built):
    """main.F90:98-99 / :116-117: accept Vd_or <- Vd_mi, Vd_mi <- Vd_pl;
    reject Vd_pl = Vd_mi = Vd_or."""
    cfg, mesh, k, o = _disch(1, 0.25)
    o.set_circuit(1.0, 2.0, 3.0)
    o.accept()
    c = o.circuit()
    assert (c["vd_pl"], c["vd_mi"], c["vd_or"]) == (1.0, 1.0, 2.0)
    o.set_circuit(1.0, 2.0, 3.0)
    o.reject()
    c = o.circuit()
    assert (c["vd_pl"], c["vd_mi"], c["vd_or"]) == (3.0, 3.0, 3.0)
