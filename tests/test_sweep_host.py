"""Host side of the batched sweep: the seeded draw of instances."""
import numpy as np

from fluidsim_gb300 import config, sweep


def test_sweep_specs_seeded_and_in_range():
    a, b = sweep.sweep_specs(192, seed=0), sweep.sweep_specs(192, seed=0)
    assert a == b and len(a) == 192
    assert {s["n"] for s in a} <= set(sweep.SIZES)
    v = np.array([s["volts"] for s in a])
    p = np.array([s["p_torr"] for s in a])
    g = np.array([s["gam"] for s in a])
    assert v.min() >= 150 and v.max() <= 400
    assert p.min() >= 0.5 and p.max() <= 10
    assert g.min() >= 0.03 and g.max() <= 0.12
    assert sweep.sweep_specs(192, seed=1) != a


def test_sweep_config_maps_the_draw():
    s = dict(n=96, volts=300.0, p_torr=2.0, gam=0.05, seed=3)
    cfg = sweep.make_config(s, mg_smooth=3)
    assert (cfg.nx, cfg.ny, cfg.mg_smooth) == (96, 96, 3)
    assert cfg.p_torr == 2.0 and cfg.gam == 0.05
    assert abs(cfg.vl * config.PH0 + 300.0) < 1e-9
