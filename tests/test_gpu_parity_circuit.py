"""Time-dependent sources on the GPU against the CPU oracle (needs a GB300):
the AC source through the RC circuit (rf = 1, circ_lib.F90:156-174, one
device kernel per stage) and the two pulse shapes (rf = 2, 3), with
electrodes on part of the wall so that the current rows carry weight.  Bars:
1e-10 per field as for the DC glow; the electrode voltage Vd_pl to 1e-12
relative and its change over the run to 1e-8 relative."""
import numpy as np
import pytest

from tests._util import field_errors

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("rf,t0,res_scale", [(1, 0.25, 1e-3), (1, 0.6, 1.0), (2, 0.1, 1.0), (3, 0.3, 1.0)])
def test_sources_vs_oracle(built, rf, t0, res_scale):
    from fluidsim_gb300 import api, config, grid
    from oracle import oracle
    cfg = config.glow(40, ny=32, rf=rf, ew=2.0, gap=10.0, lapl_rtol=1e-14)
    cfg = cfg.replace(res=cfg.res * res_scale)
    mesh = cfg.mesh()
    k = api.constants(cfg)
    st = grid.blob_state(mesh, k, noise=0.01, seed=8, vl=cfg.vl)
    gpu = api.Discharge(cfg, mesh, st)
    ref = oracle.OracleDischarge(cfg, mesh, st, solver=oracle.SOLVER_DIRECT)
    for d in (gpu, ref):
        d.set_time(t0, cfg.dt0)
    v_start = ref.circuit()["vd_pl"]
    for s in range(8):
        gi, ri = gpu.step(), ref.step()
        assert gi["lerr"] == 0 and ri["lerr"] == 0, (s, gi, ri)
        if s >= 2:
            assert gi["attempts"] == ri["attempts"], (s, gi, ri)
            assert abs(gi["dt"] - ri["dt"]) <= 1e-6 * abs(ri["dt"]), (s, gi, ri)
            assert abs(gi["idc"] - ri["idc"]) <= 1e-9 * abs(ri["idc"]), (s, gi, ri)
    e = field_errors(gpu.download(), ref.download(), k["n_zero"])
    assert max(e.values()) < 1e-10, e
    cg, cr = gpu.circuit(), ref.circuit()
    for key in ("vd_pl", "vd_mi", "vd_or", "vsrc"):
        assert abs(cg[key] - cr[key]) <= 1e-12 * abs(cr[key]) + 1e-300, (key, cg, cr)
    if rf == 1:
        moved = cr["vd_pl"] - v_start
        assert moved != 0.0
        assert abs((cg["vd_pl"] - v_start) - moved) <= 1e-8 * abs(moved), (cg, cr, v_start)
    # the ghost potentials the last stage wrote (rows with r <= ew)
    ph_g, ph_r = gpu.download()["ph"], ref.download()["ph"]
    for col in (0, -1):
        assert np.max(np.abs(ph_g[col, 1:-1] - ph_r[col, 1:-1])) <= 1e-12 * abs(cfg.vl), col

