"""Poisson solver convergence rate on the glow workload's stretched mesh.

The multigrid preconditioner over-relaxes its post-smoothing and sweeps the
electrode strips (where the mesh is stretched along x) once more after it;
without those the CG needs 10-12 iterations per step on this mesh, with them
8 (both solvers, 256^2 to 2048^2).  This test keeps that from regressing, and
runs an odd, non-square grid through the same machinery (aggregates of one
cell at the ragged edges, the FP32 levels of the FP64 solver, the one-CTA
coarse levels).  On that grid the square domain makes every cell ~3:1
(x faces conducting ~3 times better than y faces in the bulk, ~50 near the
electrodes), so the stretched "strips" span the grid, the strip sweeps are
off by design, and point smoothing needs ~15 iterations: its bound only
catches a breakdown or the iteration cap.  (Agreement of the two solvers is
tested in test_gpu_mixed.py.)"""
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("nx,ny,bound", [(256, 256, 9.0), (512, 512, 9.0), (301, 173, 24.0)])
def test_cg_iterations_per_step(built, nx, ny, bound):
    from fluidsim_gb300 import abi, api, config, grid
    cfg = config.glow(nx, ny=ny, lapl_rtol=1e-8, lapl_maxit=500)
    mesh = cfg.mesh()
    st = grid.blob_state(mesh, api.constants(cfg), noise=0.01, seed=1, vl=cfg.vl)
    for prec in (abi.FS_PREC_FP64, abi.FS_PREC_MIXED):
        d = api.Discharge(cfg.replace(precision=prec), mesh, st)
        s0 = d.run(2)   # start-up steps
        s1 = d.run(6)
        iters = (s1["lapl_iters"] - s0["lapl_iters"]) / (s1["steps"] - s0["steps"])
        assert iters <= bound, (prec, iters)
        assert s1["lapl_rejects"] == s0["lapl_rejects"], (prec, s1)
        assert s1["last_lapl_iters"] > 0 and s1["lapl_relres"] <= 1e-8, (prec, s1)
