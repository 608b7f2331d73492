"""The table-driven FP64 logarithm and exponential of the FP64 kernels
(fs_fastmath.cuh) against CUDA's log and exp on the same GPU, over the
argument ranges the kernels use and beyond (needs a GB300): within 2 ulp, and
the out-of-range arguments (zero, negative, subnormal, infinite, NaN; |x| >=
700) handed to CUDA's functions unchanged."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _eval(fn, x):
    from fluidsim_gb300 import api, abi
    lib = api.load_library()
    x = np.ascontiguousarray(x, dtype=np.float64)
    y = np.empty_like(x)
    rc = lib.fs_math_eval(fn, abi.dptr(x), abi.dptr(y), x.size)
    assert rc == 0, rc
    return y


def _ulps(a, b):
    """|a - b| in units of the last place of b."""
    sp = np.spacing(np.abs(b))
    return np.abs(a - b) / sp


def test_log_within_2ulp(built):
    rng = np.random.default_rng(5)
    x = np.concatenate([
        np.exp(rng.uniform(np.log(1e-3), np.log(1e3), 400_000)),    # mean energies in eV
        rng.uniform(0.5, 2.0, 200_000),                               # near 1 (ln x small)
        np.exp(rng.uniform(-700, 700, 200_000)),
        1.0 + np.arange(-2000, 2001) * 2.0 ** -52,                    # ln x tiny, both signs
        np.array([1.0, 2.0, 0.5, np.nextafter(2.0, 0), 2.2250738585072014e-308, 1.7e308])])
    got, ref = _eval(0, x), _eval(2, x)
    err = _ulps(got, ref)
    assert np.all(np.isfinite(got))
    assert err.max() <= 2.0, (err.max(), x[err.argmax()])


def test_exp_within_2ulp(built):
    rng = np.random.default_rng(6)
    x = np.concatenate([
        -rng.uniform(1e-2, 100.0, 400_000),       # the Scharfetter-Gummel arguments
        rng.uniform(-699.9, 699.9, 400_000),
        rng.uniform(-1e-3, 1e-3, 100_000),
        np.array([0.0, -0.0, -100.0, 1.0, -1.0, 699.0, -699.0])])
    got, ref = _eval(1, x), _eval(3, x)
    err = _ulps(got, ref)
    assert err.max() <= 2.0, (err.max(), x[err.argmax()])


def test_out_of_range_arguments_follow_cuda(built):
    x = np.array([0.0, -0.0, -1.0, 5e-324, 1e-310, np.inf, -np.inf, np.nan, 700.0, -700.0, 800.0, -800.0])
    for fn in (0, 1):
        got, ref = _eval(fn, x), _eval(fn + 2, x)
        assert np.array_equal(got, ref, equal_nan=True), (fn, got, ref)
