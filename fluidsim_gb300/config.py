"""Run configurations: the reference defaults and the 2D argon DC glow workloads.

Units are the reference's nondimensional ones (props.F90:33-37): lengths in
x0 = 1e-4 m, time in t0 = 1e-6 s, potential in ph0 = e/(eps0 x0) volts,
densities in x0**-3.  Those three scales are REAL(4) literals in the
reference, which is why they are rounded through float32 here.
"""
import dataclasses

import numpy as np

from . import abi
from .grid import make_mesh

_f = np.float32
X0 = float(_f(1e-4))
T0 = float(_f(1e-6))
E_CHARGE = float(_f(1.60217646e-19))
EPS0 = float(_f(8.85418782e-12))
PH0 = E_CHARGE / (EPS0 * X0)


@dataclasses.dataclass
class RunConfig:
    nx: int = 64
    ny: int = 64
    nspecies: int = 3
    coef_mode: int = abi.FS_COEF_TABLE
    cyl: int = 0
    rf: int = 0
    adaptive: int = 1
    precision: int = abi.FS_PREC_FP64
    lapl_maxit: int = 400
    table_n: int = 200
    mg_smooth: int = 2
    table_emin_ev: float = 0.1
    table_emax_ev: float = 50.0
    kir_arrh_a: float = 2.3e-14
    kir_arrh_e: float = 15.8
    p_torr: float = 1.0
    tg_k: float = 300.0
    gam: float = 0.07
    n_init: float = float(_f(1e11)) * X0 ** 3
    l: float = float(_f(1e-2)) / X0
    w: float = float(_f(1e-2)) / X0
    ew: float = float(_f(1e-2)) / X0      # electrode over the whole wall
    gap: float = 2.0 * float(_f(1e-2)) / X0
    vl: float = -250.0 / PH0
    res: float = 1e4 * E_CHARGE / (PH0 * T0)
    abs_tol: float = 1e-3
    rel_tol: float = 1e-4
    dt_min: float = 1.1e-12
    lapl_rtol: float = 1e-10
    # caller-side set-up (not part of fs_config)
    mesh_law: str = "geometric"
    mesh_ratio: float = 1.05
    mesh_cap: float = 4.0
    rwall: bool = False                  # dielectric upper wall (type_y = 3) instead of Neumann
    dt0: float = 1e-12 / T0

    def c_struct(self):
        c = abi.FsConfig()
        c.abi_version = abi.FS_ABI_VERSION
        for name, _ in abi.FsConfig._fields_:
            if name == "abi_version":
                continue
            setattr(c, name, getattr(self, name))
        return c

    def mesh(self):
        return make_mesh(self.nx, self.ny, self.l, self.w, self.ew, self.gap,
                         self.mesh_law, self.mesh_ratio, self.mesh_cap, self.rwall)

    def replace(self, **kw):
        return dataclasses.replace(self, **kw)

    # -- JSON files: every field by name; a file may name a subset, the rest
    # keeps its default (the reference takes its run parameters as CLI pairs,
    # main.F90:172-248, and its physics as compile-time constants)
    def to_json(self, path=None):
        import json
        text = json.dumps(dataclasses.asdict(self), indent=1, sort_keys=True)
        if path:
            with open(path, "w") as f:
                f.write(text + "\n")
        return text

    @classmethod
    def from_json(cls, src):
        """A RunConfig from a JSON file path or a JSON string; unknown keys are an error."""
        import json
        import os
        if isinstance(src, str) and os.path.exists(src):
            with open(src) as f:
                d = json.load(f)
        else:
            d = json.loads(src)
        names = {fl.name for fl in dataclasses.fields(cls)}
        unknown = sorted(set(d) - names)
        if unknown:
            raise ValueError("unknown configuration keys: %s" % ", ".join(unknown))
        return cls(**d)


def glow(n=64, **kw):
    """2D Cartesian argon DC glow: square 1 cm gap, n x n nodes, 1 Torr, 300 K,
    cathode at x = 0 at -250 V against a grounded anode, Neumann side walls,
    gamma = 0.07, three species, 200-point rate table 0.1-50 eV with Arrhenius
    ionisation 2.3e-14 exp(-15.8/eps) m^3/s, geometric 1.05 mesh toward both
    electrodes, RK-Merson rel tol 1e-4, Poisson to 1e-10.

    The first dt is 1e-12 s on grids up to 64x64 and shrinks as 64/n above:
    electrons drift ~13 um per ps in the initial field (mue ~ 530 m^2/Vs at
    1 eV, 1 Torr), so 1e-12 s exceeds the drift CFL limit of the smallest
    cell above ~128x128 and the first RK attempt overflows before the
    controller can react (the reference does the same)."""
    cfg = RunConfig(nx=n, ny=n, dt0=1e-12 / T0 * min(1.0, 64.0 / n))
    return cfg.replace(**kw)


def reference_defaults(nx=40, ny=40):
    """The reference's compile-time physics (p = 10 Torr, gamma = 0.1,
    4 species, polynomial fits, RK tolerances 1e-3) on a Cartesian uniform
    grid with whole-wall electrodes."""
    return RunConfig(nx=nx, ny=ny, nspecies=4, coef_mode=abi.FS_COEF_FITS,
                     p_torr=10.0, gam=0.10, abs_tol=1e-3, rel_tol=1e-3,
                     mesh_law="uniform", dt0=5.0e-6)
