"""ctypes front end of the CPU oracle (TEST INFRASTRUCTURE).

Only tests/, __graft_entry__.smoke() and bench.py's CPU legs import this
module.  It exposes the oracle through the same ``Handle`` interface as the
CUDA library so that a parity test drives both identically.
"""
import ctypes as C
import os
import subprocess

import numpy as np

from fluidsim_gb300 import abi
from fluidsim_gb300.api import FluidsimError, Handle

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "liboracle.so")
# the same source built for speed (-O3, contraction allowed): the timed CPU
# baseline; parity tests use LIB
LIB_TIMED = os.path.join(HERE, "liboracle_timed.so")
SOLVER_DIRECT = 0
SOLVER_BICGSTAB = 1
_libs = {}


def build(quiet=True):
    """Compile liboracle.so and liboracle_timed.so with the Makefile beside this file."""
    out = subprocess.run(["make", "-C", HERE, "all"], capture_output=True, text=True)
    if out.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + out.stdout + out.stderr)
    if not quiet:
        print(out.stdout)
    return LIB


def load(timed=False):
    """The parity build, or with timed=True the build the CPU baseline times."""
    if timed in _libs:
        return _libs[timed]
    path = LIB_TIMED if timed else LIB
    if not os.path.exists(path):
        build()
    lib = C.CDLL(path)
    abi.declare_api(lib, "or_")
    P = C.POINTER
    dp = P(C.c_double)
    lib.or_create.argtypes = [P(abi.FsConfig), P(abi.FsMesh), C.c_int32, P(C.c_void_p)]
    lib.or_create.restype = C.c_int
    lib.or_set_threads.argtypes = [C.c_int32]
    lib.or_set_threads.restype = C.c_int
    lib.or_download_k.argtypes = [C.c_void_p, dp, dp, dp, dp, C.c_int32]
    lib.or_download_k.restype = C.c_int
    lib.or_lapl_assemble.argtypes = [C.c_void_p, C.c_double, dp, dp]
    lib.or_lapl_assemble.restype = C.c_int
    lib.or_get_flux.argtypes = [C.c_double] * 2 + [C.c_int32] + [C.c_double] * 4
    lib.or_get_flux.restype = C.c_double
    lib.or_dfdph.argtypes = [C.c_double] * 2 + [C.c_int32] + [C.c_double] * 5
    lib.or_dfdph.restype = C.c_double
    lib.or_coef.argtypes = [C.c_void_p, C.c_int32, C.c_double]
    lib.or_coef.restype = C.c_double
    _libs[timed] = lib
    return lib


def set_threads(n, timed=False):
    return load(timed).or_set_threads(int(n))


def get_flux(E, dh, q, mu, D, nl, nr):
    return load().or_get_flux(E, dh, q, mu, D, nl, nr)


def dfdph(E_pl, E_mi, q, mu, D, dx, n1, n2):
    return load().or_dfdph(E_pl, E_mi, q, mu, D, dx, n1, n2)


class OracleDischarge(Handle):
    prefix = "or_"

    def __init__(self, cfg, mesh=None, state=None, solver=SOLVER_DIRECT, timed=False):
        lib = load(timed)
        mesh = mesh or cfg.mesh()
        self._c_cfg = cfg.c_struct()
        self._c_mesh = mesh.c_struct()
        ctx = C.c_void_p()
        rc = lib.or_create(C.byref(self._c_cfg), C.byref(self._c_mesh), int(solver), C.byref(ctx))
        if rc != abi.FS_OK:
            raise FluidsimError(rc, lib.or_last_error(None).decode())
        super().__init__(lib, ctx, cfg, mesh)
        self.set_time(0.0, cfg.dt0)
        if state is not None:
            self.upload(state)

    def download_k(self):
        shp = (self.nx + 2, self.ny + 2, 5)
        out = {k: np.zeros(shp, order="F") for k in ("ki", "ke", "kt", "km")}
        self.check(self._lib.or_download_k(self.ctx, *[abi.dptr(out[k]) for k in ("ki", "ke", "kt", "km")],
                                           self.nx + 2))
        return out

    def assemble(self, dt):
        n = self.nx * self.ny
        b = np.zeros(n)
        a5 = np.zeros(5 * n)
        rc = self._lib.or_lapl_assemble(self.ctx, dt, abi.dptr(b), abi.dptr(a5))
        self.check(rc)
        return b, a5.reshape(n, 5)

    def coef(self, which, T):
        return self._lib.or_coef(self.ctx, int(which), float(T))
