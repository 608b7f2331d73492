"""ctypes mirror of the POD structs in include/fluidsim_gpu.h.

The field order and types must match the header exactly; tests/test_abi.py
checks the sizes against the compiled library.
"""
import ctypes as C

FS_ABI_VERSION = 1

FS_OK = 0
FS_ERR_INVALID = -1
FS_ERR_CUDA = -2
FS_ERR_NAN = -3
FS_ERR_NEG_DENSITY = -4
FS_ERR_MIN_DT = -5
FS_ERR_NOT_CONVERGED = -6
FS_ERR_UNSUPPORTED = -7
FS_ERR_NOMEM = -8
FS_ERR_NO_DEVICE = -9

ERROR_NAMES = {
    FS_OK: "FS_OK", FS_ERR_INVALID: "FS_ERR_INVALID", FS_ERR_CUDA: "FS_ERR_CUDA",
    FS_ERR_NAN: "FS_ERR_NAN", FS_ERR_NEG_DENSITY: "FS_ERR_NEG_DENSITY",
    FS_ERR_MIN_DT: "FS_ERR_MIN_DT", FS_ERR_NOT_CONVERGED: "FS_ERR_NOT_CONVERGED",
    FS_ERR_UNSUPPORTED: "FS_ERR_UNSUPPORTED", FS_ERR_NOMEM: "FS_ERR_NOMEM",
    FS_ERR_NO_DEVICE: "FS_ERR_NO_DEVICE",
}

FS_COEF_FITS = 0
FS_COEF_TABLE = 1
FS_PREC_FP64 = 0
FS_PREC_MIXED = 1

COEF_ROWS = ("mue", "De", "k_ir", "k_ex", "nu", "beta", "k_sc", "k_si")


class FsConfig(C.Structure):
    _fields_ = [
        ("abi_version", C.c_int32), ("nx", C.c_int32), ("ny", C.c_int32),
        ("nspecies", C.c_int32), ("coef_mode", C.c_int32), ("cyl", C.c_int32),
        ("rf", C.c_int32), ("adaptive", C.c_int32), ("precision", C.c_int32),
        ("lapl_maxit", C.c_int32), ("table_n", C.c_int32), ("mg_smooth", C.c_int32),
        ("table_emin_ev", C.c_double), ("table_emax_ev", C.c_double),
        ("kir_arrh_a", C.c_double), ("kir_arrh_e", C.c_double),
        ("p_torr", C.c_double), ("tg_k", C.c_double), ("gam", C.c_double),
        ("n_init", C.c_double), ("l", C.c_double), ("w", C.c_double),
        ("ew", C.c_double), ("gap", C.c_double), ("vl", C.c_double),
        ("res", C.c_double), ("abs_tol", C.c_double), ("rel_tol", C.c_double),
        ("dt_min", C.c_double), ("lapl_rtol", C.c_double),
    ]


class FsMesh(C.Structure):
    _fields_ = [
        ("dx", C.POINTER(C.c_double)), ("dlx", C.POINTER(C.c_double)),
        ("dy", C.POINTER(C.c_double)), ("dly", C.POINTER(C.c_double)),
        ("r", C.POINTER(C.c_double)),
        ("type_x", C.POINTER(C.c_int32)), ("type_y", C.POINTER(C.c_int32)),
    ]


_CONST_NAMES = (
    "pi", "eps0", "e", "kb", "me", "x0", "ph0", "t0", "wp02", "w2",
    "tg", "p", "ninf", "n_zero",
    "mi", "mui", "vi", "Di", "Dm", "k_r", "k_mp", "k_2q", "k_3q",
    "h_ir", "h_ex", "h_si", "h_sc", "gam", "nmin_nt", "cap",
)


class FsConstants(C.Structure):
    _fields_ = [(n, C.c_double) for n in _CONST_NAMES]

    def as_dict(self):
        return {n: getattr(self, n) for n in _CONST_NAMES}


class FsStats(C.Structure):
    _fields_ = [
        ("t", C.c_double), ("dt", C.c_double), ("t_m", C.c_double),
        ("ida", C.c_double), ("idc", C.c_double), ("err_cur", C.c_double),
        ("lapl_relres", C.c_double),
        ("steps", C.c_int64), ("attempts", C.c_int64), ("rk_rejects", C.c_int64),
        ("lapl_rejects", C.c_int64), ("lapl_iters", C.c_int64),
        ("last_lapl_iters", C.c_int32), ("lerr", C.c_int32), ("dt_step", C.c_double),
    ]

    def as_dict(self):
        return {n: getattr(self, n) for n, _ in self._fields_}


def dptr(a):
    """double* of a contiguous float64 numpy array (None passes NULL)."""
    if a is None:
        return None
    return a.ctypes.data_as(C.POINTER(C.c_double))


def iptr(a):
    if a is None:
        return None
    return a.ctypes.data_as(C.POINTER(C.c_int32))


def declare_api(lib, prefix):
    """Declare argtypes/restypes of the fs_* (or or_*) entry points on lib."""
    P = C.POINTER
    dp = P(C.c_double)
    ip = P(C.c_int32)
    vp = C.c_void_p
    sig = {
        "get_constants": ([P(FsConfig), P(FsConstants)], C.c_int),
        "build_table": ([P(FsConfig), dp], C.c_int),
        "destroy": ([vp], None),
        "last_error": ([vp], C.c_char_p),
        "set_time": ([vp, C.c_double, C.c_double], C.c_int),
        "upload_state": ([vp, dp, dp, dp, dp, dp, C.c_int32, C.c_int32], C.c_int),
        "download_state": ([vp, dp, dp, dp, dp, dp, C.c_int32, C.c_int32], C.c_int),
        "ptcl_step": ([vp, dp, dp, dp, dp, ip], C.c_int),
        "lapl_solve": ([vp, C.c_double, ip, ip, dp], C.c_int),
        "accept": ([vp], C.c_int),
        "reject": ([vp], C.c_int),
        "run": ([vp, C.c_int32, P(FsStats)], C.c_int),
        "get_stats": ([vp, P(FsStats)], C.c_int),
        "get_surface_charge": ([vp, dp, dp, dp], C.c_int),
        "set_surface_charge": ([vp, dp, dp, dp], C.c_int),
        "get_controller": ([vp, dp, P(C.c_int64)], C.c_int),
        "set_controller": ([vp, C.c_double, C.c_int64], C.c_int),
        "get_circuit": ([vp, dp], C.c_int),
        "set_circuit": ([vp, dp], C.c_int),
    }
    # the Poisson warm-start vector: the GPU library only (the oracle's
    # solvers start from zero)
    optional = {
        "get_lapl_guess": ([vp, dp, C.c_int32], C.c_int),
        "set_lapl_guess": ([vp, dp, C.c_int32], C.c_int),
    }
    for name, (args, res) in sig.items():
        f = getattr(lib, prefix + name)
        f.argtypes = args
        f.restype = res
    for name, (args, res) in optional.items():
        if hasattr(lib, prefix + name):
            f = getattr(lib, prefix + name)
            f.argtypes = args
            f.restype = res
    return lib
