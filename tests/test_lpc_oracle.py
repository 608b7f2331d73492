"""CPU oracle of the learned preconditioner's network: its FP64 gradient
against central finite differences, and the BF16 rounding it emulates."""
import numpy as np
import pytest

from oracle import lpc_ref


def test_bf16_rounding():
    x = np.array([1.0, 1.00390625, 1.005859375, 3.0e-39, -2.5, 65504.0, np.inf], dtype=np.float32)
    r = lpc_ref.bf16(x)
    # representable values stay, halfway cases go to even, signs and inf kept
    assert r[0] == 1.0 and r[1] == 1.0 and r[2] == 1.0078125
    assert r[4] == -2.5 and np.isinf(r[6])
    # every result has a zero low half
    assert np.all((r.view(np.uint32) & 0xFFFF) == 0)


def test_layout_counts():
    _, n = lpc_ref.layout()
    assert 200_000 < n < 300_000


@pytest.mark.parametrize("seed", [0, 1])
def test_fp64_gradient_matches_finite_differences(seed):
    rng = np.random.default_rng(seed)
    H = W = 8
    p = lpc_ref.init_params(seed, scale_last=1.0)
    lay, _ = lpc_ref.layout()
    for l, (wo, bo) in enumerate(lay):   # nonzero biases: no ReLU input sits exactly on the kink
        co = lpc_ref.LAYERS[l][2]
        p[bo:bo + co] = 0.05 * rng.standard_normal(co)
    x0 = np.zeros((2, H, W, lpc_ref.CIN0))
    x0[..., :lpc_ref.NFEAT] = rng.standard_normal((2, H, W, lpc_ref.NFEAT))
    tgt = rng.standard_normal((2, H, W))
    mask = np.ones((H, W))
    mask[-1, :] = 0
    net = lpc_ref.Net(p, use_bf16=False, dtype=np.float64)
    loss, g = net.loss_grad(x0, tgt, mask)
    # a few weights and the bias of every layer
    idx = []
    for l, (wo, bo) in enumerate(lay):
        nz = np.flatnonzero(p[wo:bo])
        idx += list(wo + rng.choice(nz, 3, replace=False)) + [bo]
    eps = 1e-8
    for i in idx:
        pp, pm = p.copy(), p.copy()
        pp[i] += eps
        pm[i] -= eps
        lp, _ = lpc_ref.Net(pp, use_bf16=False, dtype=np.float64).loss_grad(x0, tgt, mask)
        lm, _ = lpc_ref.Net(pm, use_bf16=False, dtype=np.float64).loss_grad(x0, tgt, mask)
        fd = (lp - lm) / (2 * eps)
        assert abs(fd - g[i]) <= 1e-6 * max(1.0, abs(fd)) + 1e-7, (i, fd, g[i])
