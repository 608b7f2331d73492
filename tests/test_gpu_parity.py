"""GPU path against the CPU oracle on identical seeded inputs (needs a GB300).

Tolerances: relative L-infinity per field, with the density floor n_zero as
absolute guard, <= 1e-10 after one step; phi relative to max|phi|.
"""
import numpy as np
import pytest

from tests._util import field_errors

pytestmark = pytest.mark.gpu


def _pair(built, n, ny=None, **kw):
    from fluidsim_gb300 import api, config, grid
    from oracle import oracle
    cfg = config.glow(n, ny=ny or n, **kw)
    mesh = cfg.mesh()
    k = api.constants(cfg)
    st = grid.blob_state(mesh, k, noise=0.01, seed=7)
    gpu = api.Discharge(cfg, mesh, st)
    ref = oracle.OracleDischarge(cfg, mesh, st, solver=oracle.SOLVER_DIRECT)
    return cfg, k, gpu, ref


@pytest.mark.parametrize("n,ny", [(24, 20), (64, 64), (37, 29)])
def test_one_step_fixed_dt(built, n, ny):
    cfg, k, gpu, ref = _pair(built, n, ny, adaptive=0, lapl_rtol=1e-14)
    for s in range(3):
        gi, ri = gpu.step(), ref.step()
        assert gi["lerr"] == 0 and ri["lerr"] == 0
    e = field_errors(gpu.download(), ref.download(), k["n_zero"])
    assert max(e.values()) < 1e-10, e


def test_adaptive_steps(built):
    cfg, k, gpu, ref = _pair(built, 32, 32, lapl_rtol=1e-14)
    for s in range(8):
        gi, ri = gpu.step(), ref.step()
        if s >= 2:
            assert gi["attempts"] == ri["attempts"], (s, gi, ri)
            assert abs(gi["dt"] - ri["dt"]) <= 1e-9 * abs(ri["dt"]), (s, gi, ri)
    e = field_errors(gpu.download(), ref.download(), k["n_zero"])
    assert max(e.values()) < 1e-9, e
