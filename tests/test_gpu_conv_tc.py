"""The learned preconditioner's 3x3 convolution on the tcgen05 tensor cores
(fs_conv3x3_tc: TMA-staged BF16 operands, FP32 accumulation in tensor
memory) against a float64 numpy convolution of the same BF16-rounded inputs
and weights (needs a GB300).  Covers every channel shape the network uses
(one and two sources, 16/32/64-channel chunks, multi-chunk sources), grids
narrower than the 128-pixel tile (tap tiles) and wider (halo rows, one-row
images and runs split across CTAs included), layers whose weights leave no
room for halo rows, ragged edges and batches; and the MMA-rate probe."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _bf16_bits(x):
    """Round float32 to BF16 (nearest even); return (bits uint16, values float32)."""
    u = np.ascontiguousarray(x, dtype=np.float32).view(np.uint32)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16).astype(np.uint16)
    return r, (r.astype(np.uint32) << 16).view(np.float32)


def _ref(x, w, bias):
    """x [B][H][W][cin], w [9][cout][cin] -> [B][H][W][cout], zero padding, float64."""
    B, H, W, cin = x.shape
    cout = w.shape[1]
    xp = np.zeros((B, H + 2, W + 2, cin))
    xp[:, 1:-1, 1:-1] = x
    out = np.zeros((B, H, W, cout))
    for t in range(9):
        dy, dx = t // 3 - 1, t % 3 - 1
        out += xp[:, 1 + dy:1 + dy + H, 1 + dx:1 + dx + W] @ w[t].T.astype(np.float64)
    return out + bias


def _run(B, H, W, c1, c2, cout, mode, seed=0):
    from fluidsim_gb300 import api
    lib = api.load_library()
    rng = np.random.default_rng(seed)
    x1b, x1 = _bf16_bits(rng.standard_normal((B, H, W, c1)).astype(np.float32))
    x2b, x2 = _bf16_bits(rng.standard_normal((B, H, W, c2)).astype(np.float32)) if c2 else (None, None)
    w32 = (rng.standard_normal((9, cout, c1 + c2)) / np.sqrt(9 * (c1 + c2))).astype(np.float32)
    _, wq = _bf16_bits(w32)
    bias = rng.standard_normal(cout).astype(np.float32)
    out = np.zeros((B, H, W, cout), dtype=np.float32 if mode == 0 else np.uint16)
    rc = lib.fs_conv3x3_tc(B, H, W, c1, c2, cout, x1b.ctypes.data_as(C.c_void_p),
                           x2b.ctypes.data_as(C.c_void_p) if c2 else None,
                           w32.ctypes.data_as(C.POINTER(C.c_float)), bias.ctypes.data_as(C.POINTER(C.c_float)),
                           mode, out.ctypes.data_as(C.c_void_p))
    assert rc == 0, rc
    x = np.concatenate([x1, x2], axis=-1) if c2 else x1
    ref = _ref(x.astype(np.float64), wq.reshape(9, cout, c1 + c2), bias.astype(np.float64))
    return out, ref


@pytest.mark.parametrize("B,H,W,c1,c2,cout", [
    (1, 8, 128, 16, 0, 16), (1, 16, 256, 16, 0, 32), (2, 12, 64, 32, 0, 64), (1, 33, 47, 64, 0, 64),
    (1, 20, 128, 64, 64, 64), (1, 10, 96, 64, 32, 32), (2, 9, 40, 32, 16, 16), (1, 6, 200, 128, 0, 32),
    (3, 4, 16, 16, 16, 16), (3, 7, 384, 32, 16, 48), (2, 1, 256, 64, 0, 16), (1, 3, 130, 16, 0, 128)])
def test_conv_fp32_output(built, B, H, W, c1, c2, cout):
    out, ref = _run(B, H, W, c1, c2, cout, 0)
    err = np.abs(out - ref) / (np.abs(ref) + 1.0)
    assert err.max() < 2e-5, err.max()


def test_conv_bf16_relu_output(built):
    out, ref = _run(2, 16, 128, 32, 32, 64, 1, seed=3)
    got = (out.astype(np.uint32) << 16).view(np.float32)
    r = np.maximum(ref, 0.0)
    assert np.all(got >= 0.0)
    assert np.max(np.abs(got - r) / (np.abs(r) + 1e-2)) < 1e-2   # one BF16 rounding


@pytest.mark.parametrize("H,W,c1,c2,cout", [(1024, 1024, 16, 0, 16), (256, 256, 64, 0, 64), (256, 256, 64, 64, 64),
                                            (512, 512, 64, 32, 32), (1024, 1024, 64, 0, 64)])
def test_conv_network_shapes(built, H, W, c1, c2, cout):
    """Layers of the 4-level U-Net at the 1024^2 solver grid (the first
    encoder layer, a level-2 layer, the level-2 and level-1 decoder layers
    with their skip inputs) and a 64-channel layer at the full grid (77
    GFLOP, the compute-bound case), FP32 output; the reference is evaluated
    at 4096 random output pixels to keep the CPU side short."""
    from fluidsim_gb300 import api
    lib = api.load_library()
    rng = np.random.default_rng(5)
    x1b, x1 = _bf16_bits(rng.standard_normal((1, H, W, c1), dtype=np.float32))
    x2b, x2 = _bf16_bits(rng.standard_normal((1, H, W, c2), dtype=np.float32)) if c2 else (None, None)
    w32 = (rng.standard_normal((9, cout, c1 + c2)) / np.sqrt(9 * (c1 + c2))).astype(np.float32)
    _, wq = _bf16_bits(w32)
    bias = rng.standard_normal(cout).astype(np.float32)
    out = np.zeros((1, H, W, cout), dtype=np.float32)
    rc = lib.fs_conv3x3_tc(1, H, W, c1, c2, cout, x1b.ctypes.data_as(C.c_void_p),
                           x2b.ctypes.data_as(C.c_void_p) if c2 else None,
                           w32.ctypes.data_as(C.POINTER(C.c_float)), bias.ctypes.data_as(C.POINTER(C.c_float)),
                           0, out.ctypes.data_as(C.c_void_p))
    assert rc == 0, rc
    x = np.concatenate([x1, x2], axis=-1) if c2 else x1
    xp = np.zeros((H + 2, W + 2, c1 + c2))
    xp[1:-1, 1:-1] = x[0]
    ys, xs = rng.integers(0, H, 4096), rng.integers(0, W, 4096)
    w = wq.reshape(9, cout, c1 + c2).astype(np.float64)
    ref = np.tile(bias.astype(np.float64), (4096, 1))
    for t in range(9):
        dy, dx = t // 3 - 1, t % 3 - 1
        ref += xp[ys + 1 + dy, xs + 1 + dx] @ w[t].T
    got = out[0, ys, xs]
    err = np.abs(got - ref) / (np.abs(ref) + 1.0)
    assert err.max() < 2e-5, err.max()


def test_mma_issue_rate(built):
    """fs_mma_rate, the measurement behind the convolution's roofline: SM
    cycles per back-to-back tcgen05.mma (M = 128, K = 16, BF16).  An N = 256
    instruction cannot beat the tensor peak (8192 FLOP per cycle and SM: 128
    cycles); every N gives a positive, bounded figure."""
    from fluidsim_gb300 import api
    lib = api.load_library()
    got = {}
    for n in (16, 64, 256):
        v = C.c_double()
        rc = lib.fs_mma_rate(n, C.byref(v))
        assert rc == 0, (n, rc)
        got[n] = v.value
    print("cycles per tcgen05.mma (M=128, K=16) by N:", got)
    assert all(0.0 < c < 5000.0 for c in got.values()), got
    assert got[256] >= 0.9 * 128.0, got
