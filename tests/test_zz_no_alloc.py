"""fs_max_ne_noalloc, the allocation-free form of fs_max_ne (needs a GB300).

Callers whose stepping loop may not allocate device memory after set-up
cannot use fs_max_ne, which takes its per-call scratch from the stream-ordered
allocator.  fs_max_ne_noalloc keeps that scratch in a fixed device array of
the library.  These tests call it through the C ABI and compare it with
fs_max_ne on the same context, twice in a row, check that the call leaves the
device's free memory unchanged, and that a context beyond the array's limit
is refused.  A maximum is exact, so the results must be equal.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _noalloc(lib):
    f = lib.fs_max_ne_noalloc
    f.argtypes = [C.c_void_p, C.POINTER(C.c_double)]
    f.restype = C.c_int
    return f


def _discharge(n, ny):
    from fluidsim_gb300 import api, config, grid
    cfg = config.glow(n, ny=ny)
    mesh = cfg.mesh()
    st = grid.blob_state(mesh, api.constants(cfg), noise=0.01, seed=11, vl=cfg.vl)
    return api.Discharge(cfg, mesh, st)


def test_noalloc_matches_fs_max_ne_twice(built):
    import torch
    from fluidsim_gb300 import abi, api
    lib = api.load_library()
    noalloc = _noalloc(lib)
    d = _discharge(300, 257)
    for call in range(2):
        d.run(3)                                   # a different state for each call
        ref = d.max_ne()                           # the existing entry point
        torch.cuda.synchronize()
        free0 = torch.cuda.mem_get_info()[0]
        v = C.c_double(float("nan"))
        rc = noalloc(d.ctx, C.byref(v))
        assert rc == abi.FS_OK, d.last_error()
        free1 = torch.cuda.mem_get_info()[0]
        assert v.value == ref, (call, v.value, ref)
        assert v.value == d.download(nlev=3)["ne"].max()
        assert free1 == free0                      # no device memory taken by the call
    d.close()


def test_noalloc_refuses_contexts_beyond_its_limit(built):
    from fluidsim_gb300 import abi, api, config, grid
    lib = api.load_library()
    noalloc = _noalloc(lib)
    n = 3343                                       # 3 * 3345^2 values > 2048 * 16384
    cfg = config.glow(n, mesh_law="uniform")
    x = grid.x_nodes(n, cfg.l, "uniform")
    y = grid.y_nodes(n, cfg.w)
    tx = np.zeros((n, n), dtype=np.int32, order="F")
    ty = np.zeros((n, n), dtype=np.int32, order="F")
    tx[0, :], tx[-1, :] = -2, 2
    ty[:, 0], ty[:, -1] = -1, 1
    d = api.Discharge(cfg, grid.Mesh(n, n, x, y, tx, ty))
    v = C.c_double(0.0)
    rc = noalloc(d.ctx, C.byref(v))
    assert rc == abi.FS_ERR_INVALID
    assert "limit" in d.last_error()
    d.close()
