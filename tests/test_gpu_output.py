"""The reference's output files written from device state (needs a GB300):
read back the way the reference's save.py reads them, they hold the
downloaded fields in the reference's units, one record per call, each the
state at its call although the files are written while stepping goes on."""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("species", [3, 4])
def test_output_files_match_state(built, tmp_path, species):
    """Three species (the glow workload; f5 zeros) and four (the reference's
    defaults, fits; f5 the metastables in m^-3)."""
    from fluidsim_gb300 import api, config, grid
    cfg = config.glow(40, ny=32) if species == 3 else config.reference_defaults(40, 32)
    mesh = cfg.mesh()
    k = api.constants(cfg)
    st = grid.blob_state(mesh, k, noise=0.01, seed=2, vl=cfg.vl if species == 3 else None)
    if species == 4:
        st["nm"] = np.asfortranarray(0.1 * st["ni"])
    d = api.Discharge(cfg, mesh, st)
    d.write_output(str(tmp_path), init=True)
    states, times = [], []
    for _ in range(3):
        d.step()
        # the record is queued; the download and the next steps run while the
        # writer thread appends it, and it must hold the state of this call
        d.write_output(str(tmp_path))
        states.append(d.download())
        times.append(d.t)
    d.step()
    d.output_wait()
    rd = lambda n: np.fromfile(os.path.join(tmp_path, n), dtype=float)
    x, y, t = rd("meshx.dat"), rd("meshy.dat"), rd("time.dat")
    nx, ny, nt = len(x), len(y), len(t)
    assert (nx, ny, nt) == (40, 32, 3)
    assert np.allclose(x, mesh.x[1:-1] * k["x0"], rtol=1e-13, atol=0)
    assert np.allclose(y, mesh.y[1:-1] * k["x0"], rtol=1e-13, atol=0)
    assert np.array_equal(t, np.array(times))
    x03 = k["x0"] * k["x0"] * k["x0"]
    conv = {"f1.dat": ("ph", lambda v: v * k["ph0"]), "f2.dat": ("ne", lambda v: v / x03),
            "f3.dat": ("ni", lambda v: v / x03), "f4.dat": ("nt", lambda v: v / x03 * k["ph0"] / 1.5)}
    if species == 4:
        conv["f5.dat"] = ("nm", lambda v: v / x03)
    for fname, (field, f) in conv.items():
        data = rd(fname).reshape([nt, ny, nx])
        for r in range(nt):
            want = f(np.asarray(states[r][field])[1:-1, 1:-1]).T
            assert np.array_equal(data[r], want), (fname, r)
    assert rd("f5.dat").size == nt * ny * nx
    if species == 3:
        assert np.all(rd("f5.dat") == 0)
    for n in ("vd.dat", "ida.dat", "idc.dat", "dt.dat", "flx.dat"):
        assert rd(n).size == nt
    if species == 3:
        assert np.allclose(rd("vd.dat"), cfg.vl * k["ph0"])
