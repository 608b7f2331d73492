"""Learned Poisson preconditioner on the GPU (needs a GB300): the tensor-core
forward and backward passes against the CPU oracle (oracle/lpc_ref.py, with
the same BF16 roundings), training on harvested pairs, and the solver with
the network in the loop."""
import json

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _mixed(n, **kw):
    from fluidsim_gb300 import abi, api, config, grid
    cfg = config.glow(n, lapl_rtol=1e-8, precision=abi.FS_PREC_MIXED, **kw)
    mesh = cfg.mesh()
    k = api.constants(cfg)
    st = grid.blob_state(mesh, k, noise=0.01, seed=3, vl=cfg.vl)
    return cfg, mesh, st


def _rel(a, b):
    return float(np.linalg.norm(np.ravel(a) - np.ravel(b)) / max(np.linalg.norm(np.ravel(b)), 1e-30))


def test_lpc_forward_and_gradient_match_oracle(built):
    from fluidsim_gb300 import api
    from oracle import lpc_ref
    cfg, mesh, st = _mixed(40)
    d = api.Discharge(cfg, mesh, st)
    d.lpc_init(crop=0, max_batch=2, max_samples=4, seed=0)
    info = d.lpc_info()
    h, w = info["h"], info["w"]
    assert (h, w) == (40, 40)
    rng = np.random.default_rng(5)
    p = lpc_ref.init_params(3, scale_last=1.0)
    lay, n = lpc_ref.layout()
    assert n == info["nparam"]
    for l, (wo, bo) in enumerate(lay):
        co = lpc_ref.LAYERS[l][2]
        p[bo:bo + co] = 0.05 * rng.standard_normal(co)
    p32 = p.astype(np.float32)
    d.lpc_weights(p32)
    assert np.array_equal(d.lpc_weights(), p32)
    feat = rng.standard_normal((2, h, w, 4)).astype(np.float32)
    tgt = rng.standard_normal((2, h, w)).astype(np.float32)
    mask = np.ones((h, w), dtype=np.float32)
    mask[:, -3:] = 0
    loss, g, pred = d.lpc_grad(feat, tgt, mask)

    net = lpc_ref.Net(p32.astype(np.float64), use_bf16=True, dtype=np.float32)
    x0 = np.zeros((2, h, w, lpc_ref.CIN0), dtype=np.float32)
    x0[..., :4] = feat
    rloss, rg = net.loss_grad(x0, tgt, mask)
    rpred = net.A["y"][..., 0]
    # BF16 operands: FP32 accumulation order differs, so a rounding may land on
    # the other BF16 neighbour now and then; the bars allow for that
    assert _rel(pred, rpred) < 1e-2
    assert abs(loss - rloss) < 1e-2 * abs(rloss)
    for l, (wo, bo) in enumerate(lay):
        co = lpc_ref.LAYERS[l][2]
        assert _rel(g[wo:bo], rg[wo:bo]) < 3e-2, (l, _rel(g[wo:bo], rg[wo:bo]))
        assert _rel(g[bo:bo + co], rg[bo:bo + co]) < 3e-2, l


def test_lpc_training_and_solver(built):
    """Harvest pairs from a 256^2 run, train on crops, then solve the following
    steps with and without the network: every solve converges to lapl_rtol
    with the residual judged in FP64, the trained network fits the second
    V-cycle's correction, and with it the CG takes fewer iterations at the
    same residual.  Every solve here starts from zero (the warm-start vector
    is cleared before each step): the network's gain is measured on the
    solve it was trained for, 7 iterations per step against 8, the network
    never switched off.  (From the warm start of a developing discharge both
    take 6.)"""
    from fluidsim_gb300 import api
    cfg, mesh, st = _mixed(256)
    d = api.Discharge(cfg, mesh, st)
    d.lpc_init(crop=128, max_batch=8, max_samples=32, seed=1)
    for s in range(12):
        assert d.step()["lerr"] == 0
        if s >= 2:
            d.lpc_harvest(per_solve=4)
    assert d.lpc_info()["samples"] == 32
    hist = d.lpc_train(iters=300, batch=8, lr=1e-3, seed=2)
    assert np.all(np.isfinite(hist))
    assert hist[-30:].mean() < 0.5 * hist[:30].mean(), (hist[:30].mean(), hist[-30:].mean())
    w = d.lpc_weights()
    state = d.download(nlev=3)
    t, dt, ts = d.t, d.dt, d.ts
    runs = {}
    for use in (False, True):
        e = api.Discharge(cfg, mesh, None)
        e.upload(state)
        e.set_time(t, dt)
        e.ts = ts
        e.lpc_init(crop=0, max_batch=1, max_samples=1, seed=0)
        e.lpc_weights(w)
        e.lpc_use(2 if use else 0)
        its, offs = [], []
        for _ in range(6):
            e.set_lapl_guess(np.zeros((cfg.nx + 2, cfg.ny + 2), order="F"))
            info = e.step()
            assert info["lerr"] == 0 and info["relres"] <= cfg.lapl_rtol, info
            its.append(info["iters"])
            offs.append(e.lpc_info()["off"])
        runs[use] = its
        if use:
            runs["switched_off"] = offs
        e.close()
    print(json.dumps({"loss_first30": float(hist[:30].mean()), "loss_last30": float(hist[-30:].mean()),
                      "cg_iters_plain": runs[False], "cg_iters_network": runs[True],
                      "network_switched_off": runs["switched_off"]}))
    assert sum(runs[True]) < sum(runs[False]), runs
    assert not any(runs["switched_off"]), runs
