"""Batch driver on the GPU (needs a GB300): discharges advanced concurrently by
fs_batch_run end bit-identical to the same discharges advanced one by one
(every reduction is fixed-order, and contexts share nothing)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_batched_equals_sequential(built):
    from fluidsim_gb300 import abi, api, sweep
    specs = [dict(n=n, volts=v, p_torr=p, gam=g, seed=i)
             for i, (n, v, p, g) in enumerate([(64, 250.0, 1.0, 0.07), (96, 320.0, 3.0, 0.1),
                                               (128, 180.0, 0.7, 0.05), (64, 390.0, 8.0, 0.12),
                                               (96, 210.0, 1.5, 0.04), (128, 280.0, 5.0, 0.09)])]
    for prec in (abi.FS_PREC_FP64, abi.FS_PREC_MIXED):
        a = sweep.make_discharges(specs, prec)
        b = sweep.make_discharges(specs, prec)
        stats, rcs = api.batch_run(a, 8, nthreads=6)
        assert rcs == [0] * len(specs)
        for d in b:
            d.run(8)
        for i, (x, y) in enumerate(zip(a, b)):
            fx, fy = x.download(), y.download()
            for f in ("ni", "ne", "nt", "ph"):
                assert np.array_equal(fx[f], fy[f]), (prec, i, f)
            assert stats[i]["steps"] == 8 and x.t == y.t
        sweep.close(a)
        sweep.close(b)


def test_fused_batch_equals_sequential(built):
    """fs_batch_run_fused -- one launch per RK stage over every discharge's
    tiles, per-discharge dt and accept/reject -- ends bit-identical to the
    same discharges advanced one by one, over enough steps that some RK
    attempts are rejected and retried; discharges with different stage tile
    shapes share the batch (one launch per shape and stage)."""
    from fluidsim_gb300 import abi, api, sweep
    specs = [dict(n=n, volts=v, p_torr=p, gam=g, seed=i)
             for i, (n, v, p, g) in enumerate([(64, 250.0, 1.0, 0.07), (96, 320.0, 3.0, 0.1),
                                               (128, 180.0, 0.7, 0.05), (64, 390.0, 8.0, 0.12),
                                               (192, 210.0, 1.5, 0.04), (37, 280.0, 5.0, 0.09)])]
    a = sweep.make_discharges(specs, abi.FS_PREC_FP64)
    b = sweep.make_discharges(specs, abi.FS_PREC_FP64)
    for i, tile in ((1, (32, 4)), (3, (32, 4)), (4, (64, 4))):
        a[i].set_stage_tile(*tile)
        b[i].set_stage_tile(*tile)
    stats, rcs = api.batch_run(a, 20, nthreads=4, fused=True)
    assert rcs == [0] * len(specs)
    for d in b:
        d.run(20)
    for i, (x, y) in enumerate(zip(a, b)):
        fx, fy = x.download(nlev=3), y.download(nlev=3)
        for f in ("ni", "ne", "nt", "ph"):
            assert np.array_equal(fx[f], fy[f]), (i, f)
        sy = y.stats()
        assert stats[i]["steps"] == 20 and x.t == y.t and stats[i]["attempts"] == sy["attempts"], (i, stats[i], sy)
        assert stats[i]["rk_rejects"] == sy["rk_rejects"] and stats[i]["idc"] == sy["idc"]
    print("RK attempts rejected and retried:", sum(s["rk_rejects"] for s in stats))
    sweep.close(a)
    sweep.close(b)
