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


def test_config_json_roundtrip(tmp_path):
    from fluidsim_gb300 import config
    cfg = config.glow(48, ny=40, rf=2, rwall=True, gam=0.09)
    p = tmp_path / "run.json"
    cfg.to_json(str(p))
    back = config.RunConfig.from_json(str(p))
    assert back == cfg
    part = config.RunConfig.from_json('{"nx": 32, "ny": 16, "p_torr": 2.0}')
    assert (part.nx, part.ny, part.p_torr) == (32, 16, 2.0) and part.gam == config.RunConfig().gam
    with pytest.raises(ValueError):
        config.RunConfig.from_json('{"nx": 8, "bogus": 1}')


def test_run_log_lines(tmp_path):
    import json
    from fluidsim_gb300 import api, config, grid
    from oracle import oracle
    cfg = config.glow(12, ny=10, lapl_rtol=1e-12)
    mesh = cfg.mesh()
    st = grid.blob_state(mesh, api.constants(cfg, oracle.load(), "or_"), noise=0.01, seed=1, vl=cfg.vl)
    o = oracle.OracleDischarge(cfg, mesh, st)
    p = tmp_path / "run.jsonl"
    o.run_logged(7, str(p), every=3)
    lines = [json.loads(x) for x in open(p)]
    assert [r["step"] for r in lines] == [3, 6, 7]
    assert all(r["lerr"] == 0 and r["cg_iters"] >= 1 and r["wall_s_per_step"] > 0 for r in lines)
