"""Caller-side set-up: mesh laws, node types and seeded initial states."""
import numpy as np
import pytest

from fluidsim_gb300 import config, grid


@pytest.mark.parametrize("n", [16, 64, 256, 1024])
def test_geometric_mesh(n):
    cfg = config.glow(n)
    m = cfg.mesh()
    assert m.x[0] == 0.0 and m.x[-1] == pytest.approx(cfg.l, rel=1e-15)
    assert np.all(m.dx > 0)
    # symmetric toward both electrodes
    assert np.allclose(m.dx, m.dx[::-1], rtol=1e-12)
    ratio = m.dx[1:] / m.dx[:-1]
    half = ratio[: n // 2 - 1]
    assert np.all(half <= 1.05 * (1 + 1e-12)) and np.all(half >= 1 - 1e-12)
    assert m.dx.max() / m.dx.min() <= cfg.mesh_cap * (1 + 1e-12)
    if n >= 64:
        assert m.dx.max() / m.dx.min() == pytest.approx(cfg.mesh_cap, rel=1e-9)
    assert np.allclose(m.dlx, 0.5 * (m.dx[1:] + m.dx[:-1]))
    # y uniform (props.F90:138-163)
    assert np.allclose(m.dy, cfg.w / (n + 1), rtol=1e-12)


def test_reference_uniform_and_tanh_mesh():
    x = grid.x_nodes(40, 100.0, "uniform")
    assert np.allclose(np.diff(x), 100.0 / 41, rtol=1e-12)
    xt = grid.x_nodes(40, 100.0, "tanh")
    assert xt[0] == 0.0 and xt[-1] == pytest.approx(100.0)
    d = np.diff(xt)
    assert d[0] < d[len(d) // 2] and np.allclose(d, d[::-1], rtol=1e-5)


def test_node_types_whole_wall_electrodes():
    cfg = config.glow(12, ny=8)
    m = cfg.mesh()
    tx, ty = m.type_x, m.type_y
    assert np.all(tx[0, :] == -2) and np.all(tx[-1, :] == 2)
    assert np.all(tx[1:-1, :] == 0)
    assert np.all(ty[:, 0] == -1) and np.all(ty[:, -1] == 1)
    assert np.all(ty[:, 1:-1] == 0)


def test_node_types_partial_electrode():
    # electrode only where y <= ew or y >= gap (props.F90:200-216)
    m = grid.make_mesh(10, 10, 100.0, 100.0, ew=20.0, gap=70.0, law="uniform")
    y = m.y
    for j in range(10):
        want = -2 if (y[j] <= 20.0 or y[j] >= 70.0) else -1
        assert m.type_x[0, j] == want
        assert m.type_x[-1, j] == -want


def test_blob_state_deterministic_and_bounded():
    cfg = config.glow(32)
    m = cfg.mesh()
    k = {"x0": config.X0, "ph0": config.PH0}
    a = grid.blob_state(m, k, noise=0.01, seed=5)
    b = grid.blob_state(m, k, noise=0.01, seed=5)
    c = grid.blob_state(m, k, noise=0.01, seed=6)
    for f in ("ni", "ne", "nt"):
        assert np.array_equal(a[f], b[f])
        assert not np.array_equal(a[f], c[f])
        assert a[f].flags.f_contiguous and a[f].shape == (34, 34)
    clean = grid.blob_state(m, k)
    r = a["ne"] / clean["ne"]
    assert np.all(np.abs(r - 1) <= 0.01 + 1e-15)
    # peak 1e14 m^-3 at the centre, floor 1e8 m^-3, mean energy 1 eV
    assert clean["ne"].max() <= 1e14 * config.X0 ** 3 * (1 + 1e-12)
    assert clean["ne"].min() >= 1e8 * config.X0 ** 3
    assert np.allclose(clean["nt"] / clean["ne"] * config.PH0, 1.0)


def test_uniform_pm1_range_and_mean():
    u = grid.uniform_pm1(1, 0, 200000)
    assert u.min() >= -1 and u.max() < 1
    assert abs(u.mean()) < 0.01
