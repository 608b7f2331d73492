"""Golden vectors of the coefficient fits from the reference's own Python,
for tests/test_golden_coef.py:

  * coeftest.py:18-56, getDt and getDe (the Fortran get_Dt, get_De);
  * wvgAC.py:58-86 and :104-117, mu and nu (the Fortran get_mue, get_nu).

Those scripts plot or load data at import time (matplotlib and data files,
absent here; wvgAC.py is also Python 2), so this script parses each and
executes only the named functions, unchanged, plus the module constants they
read (coeftest.py's ph0; nu's factor ninf is set to 1 so that it returns the
bare fit).  Run from
the repository root:

    python tests/golden/make_coef_golden.py /path/to/reference

It writes tests/golden/coef_fits.json: mean energies in eV, each function's
values there (the exponential of the fit polynomial, before the
nondimensional scaling), and each function's coefficients by name as the
function holds them.
"""
import ast
import json
import os
import sys

import numpy as np


def top_level_blocks(path, names):
    """Source of the named top-level functions only (wvgAC.py as a whole is
    Python 2, its functions are also valid Python 3)."""
    with open(path) as f:
        lines = f.read().split("\n")
    out, take = [], False
    for ln in lines:
        if ln and not ln[0].isspace():
            take = any(ln.startswith("def %s(" % n) for n in names)
        if take:
            out.append(ln)
    return "\n".join(out) + "\n"


def load(path, names, extra=None, whole=True):
    with open(path) as f:
        src = f.read() if whole else top_level_blocks(path, names)
    tree = ast.parse(src, path)
    keep = []
    for node in tree.body:
        if isinstance(node, ast.FunctionDef) and node.name in names:
            keep.append(node)
        elif extra and isinstance(node, ast.Assign) and all(isinstance(t, ast.Name) for t in node.targets) \
                and node.targets[0].id in extra:
            keep.append(node)
    ns = {"np": np}
    exec(compile(ast.Module(body=keep, type_ignores=[]), path, "exec"), ns)
    coefs = {}
    for node in keep:
        if isinstance(node, ast.FunctionDef):
            c = {}
            for st in node.body:
                if isinstance(st, ast.Assign) and isinstance(st.value, (ast.Constant, ast.UnaryOp)):
                    c[st.targets[0].id] = float(eval(compile(ast.Expression(st.value), path, "eval")))
            coefs[node.name] = c
    return ns, coefs


def main():
    if len(sys.argv) != 2:
        sys.exit("usage: python tests/golden/make_coef_golden.py <reference checkout>")
    ref = sys.argv[1]
    ct, ct_coefs = load(os.path.join(ref, "coeftest.py"), ("getDt", "getDe"),
                        extra=("eps0", "e", "x0", "ph0"))
    ac, ac_coefs = load(os.path.join(ref, "wvgAC.py"), ("mu", "nu"), whole=False)
    ac["ninf"] = 1.0
    ph0 = ct["ph0"]
    # both sides of the clamps (0.234 and 157 eV) and a log-spaced sweep that
    # keeps clear of mu's branch point (ln 5.119, a REAL(4) value in the Fortran)
    t_ev = np.logspace(-1.0, 2.5, 61)
    t_ev = np.unique(np.concatenate([t_ev, [0.2, 0.234, 0.5, 1.0, 5.0, 5.3, 10.0, 157.0, 200.0]]))
    t_ev = t_ev[np.abs(np.log(t_ev) - np.log(5.119)) > 1e-3]
    out = {
        "source": {"getDt": "coeftest.py:18-36", "getDe": "coeftest.py:38-56",
                   "mu": "wvgAC.py:58-86", "nu": "wvgAC.py:104-117"},
        "t_ev": t_ev.tolist(),
        "getDt": ct["getDt"](t_ev / ph0).tolist(),
        "getDe": ct["getDe"](t_ev / ph0).tolist(),
        "mu": ac["mu"](t_ev).tolist(),
        "nu": ac["nu"](t_ev).tolist(),
        "coefs": {**ct_coefs, **ac_coefs},
    }
    here = os.path.dirname(os.path.abspath(__file__))
    with open(os.path.join(here, "coef_fits.json"), "w") as f:
        json.dump(out, f, indent=1)
    print("wrote", len(t_ev), "points")


if __name__ == "__main__":
    main()
