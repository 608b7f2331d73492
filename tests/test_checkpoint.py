"""Checkpoint and restart: a context restored from another's checkpoint (the
three-level state, phi, t, dt, the PI controller's err_prev, the step counter,
the circuit and the wall charge) continues bit for bit like the original.
The reference has no restart; this is what tests and long runs need to start
from identical states.  The oracle on the CPU here; the CUDA library in the
GPU test below (needs a GB300)."""
import numpy as np
import pytest

from fluidsim_gb300 import api, config, grid


def _cfg(**kw):
    return config.glow(24, ny=20, rf=1, rwall=True, ew=2.0, gap=10.0, lapl_rtol=1e-12, **kw)


def _run(make, cfg, n1, n2):
    mesh = cfg.mesh()
    from oracle import oracle
    st = grid.blob_state(mesh, api.constants(cfg, oracle.load(), "or_"), noise=0.01, seed=12, vl=cfg.vl)
    a = make(cfg, mesh, st)
    a.set_time(0.3, cfg.dt0)
    for _ in range(n1):
        assert a.step()["lerr"] == 0
    ck = a.checkpoint()
    for _ in range(n2):
        assert a.step()["lerr"] == 0
    b = make(cfg, mesh, None)
    b.restore(ck)
    for _ in range(n2):
        assert b.step()["lerr"] == 0
    return a, b


def _same(a, b, rtol=0.0):
    da, db = a.download(nlev=3), b.download(nlev=3)
    for f in ("ni", "ne", "nt", "ph"):
        if rtol == 0.0:
            assert np.array_equal(da[f], db[f]), f
        else:
            assert np.allclose(db[f], da[f], rtol=rtol, atol=0), (f, np.max(np.abs(db[f] / da[f] - 1)))
    if rtol == 0.0:
        assert a.t == b.t and a.dt == b.dt
        assert a.controller() == b.controller()
    else:
        assert a.t == pytest.approx(b.t, rel=1e-9)
    assert a.circuit() == b.circuit()
    sa, sb = a.surface_charge(), b.surface_charge()
    for key in sa:
        assert np.array_equal(sa[key], sb[key]), key


def test_oracle_restart_is_bit_identical(built):
    from oracle import oracle
    make = lambda cfg, mesh, st: oracle.OracleDischarge(cfg, mesh, st)
    a, b = _run(make, _cfg(), 5, 5)
    assert a.controller()["err_prev"] != 1.0   # the controller has a memory to carry
    _same(a, b)


@pytest.mark.gpu
def test_gpu_restart_is_bit_identical(built):
    make = lambda cfg, mesh, st: api.Discharge(cfg, mesh, st)
    a, b = _run(make, _cfg(), 5, 5)
    _same(a, b)


@pytest.mark.gpu
def test_gpu_mixed_restart(built):
    """The mixed path restarts to its own accuracy, not bit for bit: a restored
    context rebuilds its FP32 log-density companions from the FP64 state,
    while the running one carries the companions its stage kernel wrote."""
    make = lambda cfg, mesh, st: api.Discharge(cfg, mesh, st)
    a, b = _run(make, config.glow(32, lapl_rtol=1e-8, precision=1, adaptive=0), 6, 6)
    _same(a, b, rtol=1e-5)
