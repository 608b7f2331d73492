"""Entry points of the C ABI beyond the step itself (needs a GB300)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _discharge(n, ny, seed=5):
    from fluidsim_gb300 import api, config, grid
    cfg = config.glow(n, ny=ny)
    mesh = cfg.mesh()
    st = grid.blob_state(mesh, api.constants(cfg), noise=0.01, seed=seed, vl=cfg.vl)
    return api.Discharge(cfg, mesh, st), st


@pytest.mark.parametrize("n,ny", [(24, 20), (300, 257)])
def test_max_ne_matches_host(built, n, ny):
    """fs_max_ne: maxval(ne) over every level and the ghost ring (main.F90:131)."""
    d, st = _discharge(n, ny)
    assert d.max_ne() == st["ne"].max()
    d.run(4)
    lev = d.download(nlev=3)
    assert d.max_ne() == lev["ne"].max()


def test_upload_download_roundtrip(built):
    d, st = _discharge(40, 33)
    back = d.download(nlev=3)
    for f in ("ni", "ne", "nt"):
        for lev in range(3):
            assert np.array_equal(back[f][:, :, lev], st[f])
    assert np.array_equal(back["ph"], st["ph"])


def test_errors_are_reported_not_fatal(built):
    """Bad arguments return FS_ERR_INVALID with a message; the context stays usable."""
    import ctypes as C
    from fluidsim_gb300 import abi, api
    d, st = _discharge(16, 12)
    rc = d._lib.fs_upload_state(d.ctx, None, None, None, None, None, 3, 2)
    assert rc == abi.FS_ERR_INVALID and "nlev" in d.last_error()
    d.run(3)
    assert np.isfinite(d.max_ne())
