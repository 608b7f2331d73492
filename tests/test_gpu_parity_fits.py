"""The reference's own physics on the GPU (needs a GB300): four species
(with metastables), the per-node coefficient fits of ptcl_props.F90:182-429
(FS_COEF_FITS), 10 Torr, gamma = 0.1, uniform mesh -- against the CPU oracle
on identical inputs.  Bar: 1e-10 per field (relative, density floor as
absolute guard; phi relative to max|phi|), as for the glow workload."""
import numpy as np
import pytest

from tests._util import field_errors, rel_linf

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("adaptive", [0, 1])
def test_fits_four_species_vs_oracle(built, adaptive):
    from fluidsim_gb300 import api, config, grid
    from oracle import oracle
    cfg = config.reference_defaults(40, 32).replace(lapl_rtol=1e-14, adaptive=adaptive)
    mesh = cfg.mesh()
    k = api.constants(cfg)
    st = grid.blob_state(mesh, k, noise=0.01, seed=5)
    st["nm"] = np.asfortranarray(0.1 * st["ni"])
    gpu = api.Discharge(cfg, mesh, st)
    ref = oracle.OracleDischarge(cfg, mesh, st, solver=oracle.SOLVER_DIRECT)
    for s in range(8):
        gi, ri = gpu.step(), ref.step()
        assert gi["lerr"] == 0 and ri["lerr"] == 0, (s, gi, ri)
        if s >= 2 and adaptive:
            assert gi["attempts"] == ri["attempts"], (s, gi, ri)
            assert abs(gi["dt"] - ri["dt"]) <= 1e-6 * abs(ri["dt"]), (s, gi, ri)
    g, r = gpu.download(), ref.download()
    e = field_errors(g, r, k["n_zero"])
    e["nm"] = rel_linf(g["nm"], r["nm"], k["n_zero"])
    assert max(e.values()) < 1e-10, e
