"""The oracle's coefficient fits against the reference's own Python
(tests/golden/coef_fits.json, made by tests/golden/make_coef_golden.py):
coeftest.py's getDe and getDt are the Fortran get_De (ptcl_props.F90:268-291)
and get_Dt (:293-316); wvgAC.py's mu and nu are get_mue (:194-221) and get_nu
(:376-395); all before the nondimensional scaling.

The Fortran writes the fit coefficients without a d exponent, so they are
REAL(4) literals, while the Python holds them in double.  Evaluated with the
Python's coefficients rounded to float32 the oracle agrees to 1e-11 (the
degree-11 diffusion polynomials sum terms of ~1e4 to an exponent of ~57 near
the upper clamp, so the evaluation order moves the exponent by ~1e-12);
against the Python's own values the difference is the REAL(4) rounding of
the coefficients, below 3e-4 relative."""
import json
import os

import numpy as np
import pytest

from fluidsim_gb300 import api, config
from oracle import oracle

HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.fixture(scope="module")
def golden():
    with open(os.path.join(HERE, "golden", "coef_fits.json")) as f:
        return json.load(f)


def _f32(c, names):
    return [float(np.float32(c[n])) for n in names]


def _poly(c, x):
    s = c[0] + c[1] * x
    for k in range(2, len(c)):
        s = s + c[k] * x ** k
    return s


def _fit_f32(name, coefs, x):
    """The reference's fit with its coefficients as REAL(4) literals."""
    if name == "mu":
        lo = _poly(_f32(coefs, ["a1", "b1", "c1", "d1", "f1", "g1"]), x)
        hi = _poly(_f32(coefs, ["a2", "b2", "c2", "d2", "f2", "g2"]), x)
        return np.exp(np.where(x < float(np.log(np.float32(5.119))), lo, hi))
    return np.exp(_poly(_f32(coefs, list(coefs)), x))   # a, b, c, ... in the function's order


@pytest.mark.parametrize("which,name", [(0, "mu"), (1, "getDe"), (4, "nu"), (9, "getDt")])
def test_fits_match_reference_python(built, golden, which, name):
    cfg = config.glow(8, coef_mode=0)   # the fits, not the table
    o = oracle.OracleDischarge(cfg, cfg.mesh(), None)
    k = api.constants(cfg, oracle.load(), "or_")
    x03 = k["x0"] ** 3
    scale = {"mu": k["x0"] / k["ninf"] * k["t0"] * k["ph0"], "getDe": k["x0"] / k["ninf"] * k["t0"],
             "getDt": k["x0"] / k["ninf"] * k["t0"], "nu": k["ninf"] * k["t0"] / x03}[name]
    t_ev = np.array(golden["t_ev"])
    got = np.array([o.coef(which, t / k["ph0"]) for t in t_ev]) / scale
    want = np.array(golden[name])
    assert np.max(np.abs(got / want - 1)) < 3e-4, np.max(np.abs(got / want - 1))
    x = np.log(np.maximum(0.234, np.minimum(157.0, t_ev)))
    exact = _fit_f32(name, golden["coefs"][name], x)
    assert np.max(np.abs(got / exact - 1)) < 1e-11, np.max(np.abs(got / exact - 1))
