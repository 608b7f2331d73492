"""The largest workload size (2048x2048, 4.2 M nodes; needs a GB300): the
mixed path steps adaptively, the FP64 path replays its accepted step sizes;
every Poisson solve converges to lapl_rtol, the densities stay finite and
positive, and the two agree to the mixed path's 1e-5 bar.  The CPU oracle is
out of reach at this size; the FP64 GPU path stands for it (it matches the
oracle to 1e-10 at the smaller sizes).

A fixed dt is not used here: near the electrodes the hot-electron energy
diffusion limits an explicit step to ~dx_min^2 / (4 * 5/3 * D_e), about 4e-16 s
at 2048^2, below the glow's scaled fixed step, and both precisions would
amplify their rounding differences alike (an instability, not an arithmetic
error)."""
import numpy as np
import pytest

from tests._util import field_errors
from tests.test_gpu_mixed import _replay

pytestmark = pytest.mark.gpu


def test_2048_adaptive_replay(built):
    from fluidsim_gb300 import abi, api, config, grid
    cfg = config.glow(2048, lapl_rtol=1e-8)
    mesh = cfg.mesh()
    k = api.constants(cfg)
    st = grid.blob_state(mesh, k, noise=0.01, seed=9, vl=cfg.vl)
    a = api.Discharge(cfg.replace(adaptive=0), mesh, st)
    b = api.Discharge(cfg.replace(precision=abi.FS_PREC_MIXED), mesh, st)
    _replay(a, b, 12)
    da, db = a.download(), b.download()
    for f in ("ni", "ne", "nt"):
        for d in (da, db):
            v = np.asarray(d[f])[1:-1, 1:-1]
            assert np.all(np.isfinite(v)) and v.min() > 0, f
    e = field_errors(db, da, k["n_zero"])
    assert max(e.values()) < 1e-5, e
