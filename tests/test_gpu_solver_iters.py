"""Poisson solver convergence rate on stretched and anisotropic meshes.

The multigrid preconditioner over-relaxes its post-smoothing and sweeps the
electrode strips (where the mesh is stretched along x) once more after it;
without those the CG needs 10-12 iterations per step on the glow mesh, with
them 8 (both solvers, 256^2 to 2048^2).  On a 301x173 grid the square domain
makes every cell ~3:1 (x faces conducting ~3 times better than y faces in the
bulk, ~50 near the electrodes), so the "strips" would span the grid; there
the finest level smooths with zebra x-lines instead (chosen from the mesh),
which takes the CG from 13-15 iterations per step with point smoothing to 8.
The tanh mesh at 1024^2 is stretched over more than 64 columns at each
electrode (no strip sweeps) but isotropic in the middle: point smoothing
alone takes 8-9 iterations there.  The odd grid also runs the ragged-edge
aggregates, the FP32 levels of the FP64 solver and the one-CTA coarse levels.
(Agreement of the two solvers is tested in test_gpu_mixed.py.)"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _iters(cfg, mesh, st, mode=-1):
    from fluidsim_gb300 import api
    d = api.Discharge(cfg, mesh, st)
    d.set_line_smoother(mode)
    s0 = d.run(2)   # start-up steps
    s1 = d.run(6)
    iters = (s1["lapl_iters"] - s0["lapl_iters"]) / (s1["steps"] - s0["steps"])
    assert s1["lapl_rejects"] == s0["lapl_rejects"], s1
    assert s1["last_lapl_iters"] > 0 and s1["lapl_relres"] <= 1e-8, s1
    return d, iters


@pytest.mark.parametrize("nx,ny,law,bound,xline", [(256, 256, None, 9.0, 0), (512, 512, None, 9.0, 0),
                                                   (301, 173, None, 10.0, 1), (1024, 1024, "tanh", 10.0, 0)])
def test_cg_iterations_per_step(built, nx, ny, law, bound, xline):
    from fluidsim_gb300 import abi, api, config, grid
    cfg = config.glow(nx, ny=ny, lapl_rtol=1e-8, lapl_maxit=500)
    if law:
        cfg = cfg.replace(mesh_law=law)
    mesh = cfg.mesh()
    st = grid.blob_state(mesh, api.constants(cfg), noise=0.01, seed=1, vl=cfg.vl)
    for prec in (abi.FS_PREC_FP64, abi.FS_PREC_MIXED):
        d, iters = _iters(cfg.replace(precision=prec), mesh, st)
        assert d.line_smoother() == xline, (prec, d.line_smoother())
        assert iters <= bound, (prec, iters)
        d.close()


def test_xline_and_point_smoothing_agree(built):
    """Forced x-line smoothing on the glow mesh (which chooses point sweeps
    with the strips) converges to the same relative residual, and the
    potentials of the two runs agree to the solver tolerance."""
    from fluidsim_gb300 import abi, api, config, grid
    cfg = config.glow(256, lapl_rtol=1e-10, lapl_maxit=500)
    cfg = cfg.replace(dt0=cfg.dt0 / 4)
    mesh = cfg.mesh()
    st = grid.blob_state(mesh, api.constants(cfg), noise=0.01, seed=3, vl=cfg.vl)
    for prec in (abi.FS_PREC_FP64, abi.FS_PREC_MIXED):
        a, ia = _iters(cfg.replace(precision=prec, adaptive=0), mesh, st, 0)
        b, ib = _iters(cfg.replace(precision=prec, adaptive=0), mesh, st, 1)
        assert a.line_smoother() == 0 and b.line_smoother() == 1
        assert ib <= ia + 2, (prec, ia, ib)
        pa, pb = a.download()["ph"], b.download()["ph"]
        assert np.max(np.abs(pa - pb)) <= 1e-6 * np.max(np.abs(pa)), prec
        a.close()
        b.close()
