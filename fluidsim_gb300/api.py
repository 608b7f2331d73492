"""Python front end of the C ABI, mirroring the reference's module interface.

``Discharge`` owns one fs_ctx and exposes the reference's subroutines under
their own names: ``ptcl_step`` (ptcl_lib.F90:32-97), ``lapl_solve``
(lapl_lib.F90:57-121), ``accept``/``reject`` (main.F90:83-121) and ``step``,
one iteration of the main.F90:68-121 loop.  State crosses the boundary as the
reference's Fortran-ordered arrays (nx+2, ny+2[, 3]).
"""
import ctypes as C
import os

import numpy as np

from . import abi

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_NAME = "libfluidsim_gb300.so"
_lib = None


class FluidsimError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__("%s (%d): %s" % (abi.ERROR_NAMES.get(code, "?"), code, msg))
        self.code = code


def lib_path():
    return os.path.join(_HERE, LIB_NAME)


def load_library():
    """Load the in-tree CUDA library; raise if it has not been built."""
    global _lib
    if _lib is not None:
        return _lib
    p = lib_path()
    if not os.path.exists(p):
        raise FluidsimError(abi.FS_ERR_NO_DEVICE,
                            "%s not built; run __graft_entry__.build() first" % p)
    lib = C.CDLL(p)
    abi.declare_api(lib, "fs_")
    lib.fs_create.argtypes = [C.POINTER(abi.FsConfig), C.POINTER(abi.FsMesh),
                              C.POINTER(C.c_void_p)]
    lib.fs_create.restype = C.c_int
    lib.fs_abi_version.restype = C.c_int32
    lib.fs_max_ne.argtypes = [C.c_void_p, C.POINTER(C.c_double)]
    lib.fs_max_ne.restype = C.c_int
    lib.fs_stream.argtypes = [C.c_void_p]
    lib.fs_stream.restype = C.c_void_p
    lib.fs_profile.argtypes = [C.c_void_p, C.c_int32]
    lib.fs_profile.restype = C.c_int
    lib.fs_profile_read.argtypes = [C.c_void_p, C.POINTER(C.c_double), C.POINTER(C.c_int64), C.c_int32]
    lib.fs_profile_read.restype = C.c_int
    lib.fs_launch_count.argtypes = [C.c_void_p]
    lib.fs_launch_count.restype = C.c_int64
    lib.fs_set_stage_tile.argtypes = [C.c_void_p, C.c_int32, C.c_int32]
    lib.fs_set_stage_tile.restype = C.c_int
    lib.fs_set_line_smoother.argtypes = [C.c_void_p, C.c_int32]
    lib.fs_set_line_smoother.restype = C.c_int
    lib.fs_line_smoother.argtypes = [C.c_void_p]
    lib.fs_line_smoother.restype = C.c_int
    lib.fs_fp64_rate.argtypes = [C.c_int32, C.POINTER(C.c_double)]
    lib.fs_fp64_rate.restype = C.c_int
    lib.fs_math_eval.argtypes = [C.c_int32, C.POINTER(C.c_double), C.POINTER(C.c_double), C.c_int64]
    lib.fs_math_eval.restype = C.c_int
    lib.fs_conv3x3_tc.argtypes = [C.c_int32] * 6 + [C.c_void_p, C.c_void_p, C.POINTER(C.c_float),
                                                    C.POINTER(C.c_float), C.c_int32, C.c_void_p]
    lib.fs_conv3x3_tc.restype = C.c_int
    fp, i32, vp = C.POINTER(C.c_float), C.c_int32, C.c_void_p
    for name, args in (("fs_lpc_init", [vp, i32, i32, i32, C.c_uint64]),
                       ("fs_lpc_harvest", [vp, i32, C.POINTER(i32)]),
                       ("fs_lpc_train", [vp, i32, i32, C.c_float, C.c_uint64, fp]),
                       ("fs_lpc_use", [vp, i32]),
                       ("fs_lpc_weights", [vp, fp, C.c_int64, i32]),
                       ("fs_lpc_grad", [vp, fp, fp, fp, i32, fp, fp, fp]),
                       ("fs_lpc_info", [vp, C.POINTER(i32), C.POINTER(i32), C.POINTER(i32),
                                        C.POINTER(C.c_int64), C.POINTER(i32), C.POINTER(C.c_int64),
                                        C.POINTER(C.c_int64)])):
        getattr(lib, name).argtypes = args
        getattr(lib, name).restype = C.c_int
    lib.fs_batch_run.argtypes = [C.POINTER(C.c_void_p), C.c_int32, C.c_int32, C.c_double, C.c_int32,
                                 C.POINTER(abi.FsStats), C.POINTER(C.c_int32)]
    lib.fs_batch_run.restype = C.c_int
    lib.fs_batch_run_fused.argtypes = lib.fs_batch_run.argtypes
    lib.fs_batch_run_fused.restype = C.c_int
    lib.fs_write_output.argtypes = [C.c_void_p, C.c_char_p, C.c_int32]
    lib.fs_write_output.restype = C.c_int
    lib.fs_output_wait.argtypes = [C.c_void_p]
    lib.fs_output_wait.restype = C.c_int
    _lib = lib
    return lib


def constants(cfg, lib=None, prefix="fs_"):
    lib = lib or load_library()
    out = abi.FsConstants()
    c = cfg.c_struct()
    rc = getattr(lib, prefix + "get_constants")(C.byref(c), C.byref(out))
    if rc:
        raise FluidsimError(rc, "get_constants failed")
    return out.as_dict()


def coefficient_table(cfg, lib=None, prefix="fs_"):
    lib = lib or load_library()
    out = np.zeros(8 * cfg.table_n)
    c = cfg.c_struct()
    rc = getattr(lib, prefix + "build_table")(C.byref(c), abi.dptr(out))
    if rc:
        raise FluidsimError(rc, "build_table failed")
    return out.reshape(8, cfg.table_n)


class Handle:
    """One simulation context behind an fs_* style C interface."""

    prefix = "fs_"

    def __init__(self, lib, ctx, cfg, mesh):
        self._lib = lib
        self.ctx = ctx
        self.cfg = cfg
        self.mesh = mesh
        self.nx, self.ny = cfg.nx, cfg.ny
        self.dt = cfg.dt0
        self.t = 0.0
        self.ts = 0

    def _f(self, name):
        return getattr(self._lib, self.prefix + name)

    def last_error(self):
        m = self._f("last_error")(self.ctx)
        return m.decode() if m else ""

    def check(self, rc):
        if rc != abi.FS_OK:
            raise FluidsimError(rc, self.last_error())

    def close(self):
        if self.ctx:
            self._f("destroy")(self.ctx)
            self.ctx = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # -- state ---------------------------------------------------------------
    def set_time(self, t, dt):
        self.t, self.dt = float(t), float(dt)
        self.check(self._f("set_time")(self.ctx, self.t, self.dt))

    def upload(self, state):
        """state: dict with ni, ne, nt[, nm], ph as (nx+2, ny+2) or (nx+2, ny+2, 3)."""
        ni = np.asfortranarray(state["ni"], dtype=np.float64)
        nlev = 3 if ni.ndim == 3 else 1
        arrs = [np.asfortranarray(state[k], dtype=np.float64) if state.get(k) is not None else None
                for k in ("ni", "ne", "nt", "nm", "ph")]
        self._keep = arrs
        self.check(self._f("upload_state")(self.ctx, *[abi.dptr(a) for a in arrs],
                                           self.nx + 2, nlev))

    def download(self, nlev=1, out=None):
        """The module arrays (ni, ne, nt[, nm], ph) in the reference's layout;
        into the caller's arrays when `out` holds them (Fortran-ordered float64
        of the right shapes, e.g. views of pinned memory), else new ones."""
        shp = (self.nx + 2, self.ny + 2) + ((3,) if nlev == 3 else ())
        if out is None:
            out = {k: np.zeros(shp, order="F") for k in ("ni", "ne", "nt")}
            out["nm"] = np.zeros(shp, order="F") if self.cfg.nspecies == 4 else None
            out["ph"] = np.zeros((self.nx + 2, self.ny + 2), order="F")
        else:
            out = dict(out)
            out.setdefault("nm", None)
            for k, want in (("ni", shp), ("ne", shp), ("nt", shp), ("ph", (self.nx + 2, self.ny + 2))):
                a = out[k]
                if a.shape != want or a.dtype != np.float64 or not a.flags.f_contiguous:
                    raise ValueError("download: %s must be a Fortran-ordered float64 array of shape %s" % (k, want))
            if self.cfg.nspecies == 4 and out["nm"] is None:
                out["nm"] = np.zeros(shp, order="F")
        self.check(self._f("download_state")(
            self.ctx, abi.dptr(out["ni"]), abi.dptr(out["ne"]), abi.dptr(out["nt"]),
            abi.dptr(out["nm"]), abi.dptr(out["ph"]), self.nx + 2, nlev))
        return out

    def surface_charge(self):
        """sfc_lib's sig_pl, sig_mi, sig_or (nx+2 entries each, Fortran index
        i at [i-1]): the charge of the dielectric wall (type_y == 3) nodes."""
        out = [np.zeros(self.nx + 2) for _ in range(3)]
        self.check(self._f("get_surface_charge")(self.ctx, *[abi.dptr(a) for a in out]))
        return dict(zip(("sig_pl", "sig_mi", "sig_or"), out))

    def set_surface_charge(self, sig_pl=None, sig_mi=None, sig_or=None):
        arrs = [None if a is None else np.ascontiguousarray(a, dtype=np.float64) for a in (sig_pl, sig_mi, sig_or)]
        for a in arrs:
            if a is not None and a.shape != (self.nx + 2,):
                raise ValueError("surface charge arrays have nx+2 entries")
        self.check(self._f("set_surface_charge")(self.ctx, *[abi.dptr(a) for a in arrs]))

    def controller(self):
        """ptcl_step's err_prev and main's step counter ts."""
        e, ts = C.c_double(), C.c_int64()
        self.check(self._f("get_controller")(self.ctx, C.byref(e), C.byref(ts)))
        return dict(err_prev=e.value, ts=ts.value)

    def set_controller(self, err_prev, ts):
        self.check(self._f("set_controller")(self.ctx, float(err_prev), int(ts)))
        self.ts = int(ts)

    def checkpoint(self):
        """Everything a restart needs: the three-level state, phi, time, dt,
        the controller, the circuit, the wall charge and the Poisson solver's
        warm-start vector (host copies)."""
        return dict(state=self.download(nlev=3), t=self.t, dt=self.dt, controller=self.controller(),
                    circuit=self.circuit(), surface_charge=self.surface_charge(), lapl_guess=self.lapl_guess())

    def restore(self, ck):
        self.upload(ck["state"])
        self.set_time(ck["t"], ck["dt"])
        self.set_controller(ck["controller"]["err_prev"], ck["controller"]["ts"])
        c = ck["circuit"]
        self.set_circuit(c["vd_pl"], c["vd_mi"], c["vd_or"])
        sc = ck["surface_charge"]
        self.set_surface_charge(sc["sig_pl"], sc["sig_mi"], sc["sig_or"])
        if "lapl_guess" in ck:
            self.set_lapl_guess(ck["lapl_guess"])

    def lapl_guess(self):
        """The Poisson solver's warm-start vector, (nx+2, ny+2) Fortran-ordered
        (None for a library without one: the oracle starts from zero)."""
        if not hasattr(self._lib, self.prefix + "get_lapl_guess"):
            return None
        d = np.zeros((self.nx + 2, self.ny + 2), order="F")
        self.check(self._f("get_lapl_guess")(self.ctx, abi.dptr(d), self.nx + 2))
        return d

    def set_lapl_guess(self, d):
        if d is None or not hasattr(self._lib, self.prefix + "set_lapl_guess"):
            return
        d = np.asfortranarray(d, dtype=np.float64)
        self.check(self._f("set_lapl_guess")(self.ctx, abi.dptr(d), self.nx + 2))

    def circuit(self):
        """circ_lib's Vd_pl, Vd_mi, Vd_or and the last source voltage Vsrc."""
        v = np.zeros(4)
        self.check(self._f("get_circuit")(self.ctx, abi.dptr(v)))
        return dict(zip(("vd_pl", "vd_mi", "vd_or", "vsrc"), v.tolist()))

    def set_circuit(self, vd_pl, vd_mi, vd_or):
        v = np.array([vd_pl, vd_mi, vd_or], dtype=np.float64)
        self.check(self._f("set_circuit")(self.ctx, abi.dptr(v)))

    # -- the reference's subroutines -----------------------------------------
    def ptcl_step(self):
        dt = C.c_double(self.dt)
        tm, ida, idc = C.c_double(), C.c_double(), C.c_double()
        att = C.c_int32()
        self.check(self._f("ptcl_step")(self.ctx, C.byref(dt), C.byref(tm), C.byref(ida),
                                        C.byref(idc), C.byref(att)))
        self.dt = dt.value
        return dict(dt=dt.value, t_m=tm.value, ida=ida.value, idc=idc.value,
                    attempts=att.value)

    def lapl_solve(self):
        lerr, it, rr = C.c_int32(), C.c_int32(), C.c_double()
        self.check(self._f("lapl_solve")(self.ctx, self.dt, C.byref(lerr), C.byref(it),
                                         C.byref(rr)))
        return dict(lerr=lerr.value, iters=it.value, relres=rr.value)

    def accept(self):
        self.check(self._f("accept")(self.ctx))
        self.ts += 1
        self.t += self.dt

    def reject(self):
        self.check(self._f("reject")(self.ctx))
        self.dt = self.dt / 2.0

    def step(self):
        """One iteration of the main.F90:68-121 loop through the separate calls."""
        info = {}
        if self.ts > 1:
            info.update(self.ptcl_step())
        info.update(self.lapl_solve())
        if info["lerr"] == 0:
            self.accept()
        else:
            self.reject()
        return info

    def run_logged(self, nsteps, log, every=1):
        """nsteps main-loop iterations through the separate calls, with one
        JSON line per `every` steps written to `log` (a path or a file
        object): the figures the reference prints every few seconds
        (main.F90:124-138: step, t, dt, t_m, Vd, Ida, Idc, max n_e) plus RK
        attempts, CG iterations and residual, and the wall time per step."""
        import json
        import time
        own = isinstance(log, (str, bytes, os.PathLike))
        f = open(log, "a") if own else log
        try:
            last, since = time.perf_counter(), 0
            for s in range(nsteps):
                info = self.step()
                since += 1
                if since < every and s + 1 != nsteps:
                    continue
                now = time.perf_counter()
                rec = {"step": self.ts, "t": self.t, "dt": self.dt, "lerr": info["lerr"],
                       "attempts": info.get("attempts", 0), "cg_iters": info["iters"],
                       "relres": info["relres"], "t_m": info.get("t_m"), "ida": info.get("ida"),
                       "idc": info.get("idc"), "vd": self.circuit()["vd_pl"],
                       "wall_s_per_step": (now - last) / since}
                if hasattr(self, "max_ne"):
                    rec["max_ne"] = self.max_ne()
                f.write(json.dumps(rec) + "\n")
                last, since = now, 0
            f.flush()
        finally:
            if own:
                f.close()

    def run(self, nsteps):
        """nsteps main-loop iterations inside the library (fs_run)."""
        st = abi.FsStats()
        self.check(self._f("run")(self.ctx, int(nsteps), C.byref(st)))
        d = st.as_dict()
        self.t, self.dt, self.ts = d["t"], d["dt"], d["steps"]
        return d

    def stats(self):
        st = abi.FsStats()
        self.check(self._f("get_stats")(self.ctx, C.byref(st)))
        return st.as_dict()


class Discharge(Handle):
    """A discharge simulated by the CUDA library: lapl_init + ptcl_init +
    circ_init on construction, state in device memory until downloaded."""

    prefix = "fs_"

    def __init__(self, cfg, mesh=None, state=None):
        lib = load_library()
        mesh = mesh or cfg.mesh()
        self._c_cfg = cfg.c_struct()
        self._c_mesh = mesh.c_struct()
        ctx = C.c_void_p()
        rc = lib.fs_create(C.byref(self._c_cfg), C.byref(self._c_mesh), C.byref(ctx))
        if rc != abi.FS_OK:
            msg = lib.fs_last_error(None)
            raise FluidsimError(rc, msg.decode() if msg else "fs_create failed")
        super().__init__(lib, ctx, cfg, mesh)
        self.set_time(0.0, cfg.dt0)
        if state is not None:
            self.upload(state)

    PROF_CLASSES = ("stage", "assemble", "smooth", "transfer", "bottom", "cg", "coarsen", "control")

    def stream_handle(self):
        """cudaStream_t (as an int) that all of this context's work runs on."""
        return self._lib.fs_stream(self.ctx)

    def profile(self, classes=None):
        """Time the given kernel classes (names from PROF_CLASSES; None = all,
        [] = off) with CUDA events around each launch."""
        if classes is None:
            mask = (1 << len(self.PROF_CLASSES)) - 1
        else:
            mask = 0
            for c in classes:
                mask |= 1 << self.PROF_CLASSES.index(c)
        self.check(self._lib.fs_profile(self.ctx, mask))

    def profile_read(self):
        n = len(self.PROF_CLASSES)
        ms = (C.c_double * n)()
        cnt = (C.c_int64 * n)()
        self.check(self._lib.fs_profile_read(self.ctx, ms, cnt, n))
        return {k: (ms[i], cnt[i]) for i, k in enumerate(self.PROF_CLASSES)}

    def set_stage_tile(self, bx, by):
        """RK stage kernel tile (FP64 path): (32, 8), (32, 4) or (64, 4)."""
        self.check(self._lib.fs_set_stage_tile(self.ctx, int(bx), int(by)))

    def set_line_smoother(self, mode):
        """V-cycle smoother: -1 chosen from the mesh, 0 point red-black, 1 zebra x-line."""
        self.check(self._lib.fs_set_line_smoother(self.ctx, int(mode)))

    def line_smoother(self):
        """1 while the V-cycles smooth with x-lines, 0 with points."""
        return self._lib.fs_line_smoother(self.ctx)

    def launch_count(self):
        return self._lib.fs_launch_count(self.ctx)

    def max_ne(self):
        v = C.c_double()
        self.check(self._lib.fs_max_ne(self.ctx, C.byref(v)))
        return v.value

    def write_output(self, directory, init=False):
        """The reference's output files in `directory` (see fs_write_output):
        a record is appended by a writer thread while stepping continues."""
        self.check(self._lib.fs_write_output(self.ctx, os.fsencode(directory), 1 if init else 0))

    def output_wait(self):
        """Wait until the last record is on disk."""
        self.check(self._lib.fs_output_wait(self.ctx))

    # -- learned Poisson preconditioner (mixed contexts) -----------------------
    def lpc_init(self, crop=0, max_batch=16, max_samples=64, seed=0):
        """Network on the fine grid; training on crops of crop x crop cells
        (a multiple of 8; 0: 128, at most the grid), batches up to max_batch,
        up to max_samples stored training pairs (full grids)."""
        self.check(self._lib.fs_lpc_init(self.ctx, crop, max_batch, max_samples, seed))

    def lpc_info(self):
        h, w, n, off = C.c_int32(), C.c_int32(), C.c_int32(), C.c_int32()
        npar, sol, nns = C.c_int64(), C.c_int64(), C.c_int64()
        self.check(self._lib.fs_lpc_info(self.ctx, C.byref(h), C.byref(w), C.byref(n), C.byref(npar),
                                         C.byref(off), C.byref(sol), C.byref(nns)))
        return dict(h=h.value, w=w.value, samples=n.value, nparam=npar.value, off=off.value,
                    solves=sol.value, nn_solves=nns.value)

    def lpc_harvest(self, per_solve=4):
        a = C.c_int32()
        self.check(self._lib.fs_lpc_harvest(self.ctx, per_solve, C.byref(a)))
        return a.value

    def lpc_train(self, iters, batch, lr=1e-3, seed=0):
        hist = np.zeros(max(iters, 1), dtype=np.float32)
        self.check(self._lib.fs_lpc_train(self.ctx, iters, batch, lr, seed,
                                          hist.ctypes.data_as(C.POINTER(C.c_float))))
        return hist[:iters]

    def lpc_use(self, mode=1):
        """0: plain multigrid-PCG; 1 (or True): the network where it is faster;
        2: the network in every solve."""
        self.check(self._lib.fs_lpc_use(self.ctx, int(mode)))

    def lpc_weights(self, w=None):
        """Get the FP32 parameters, or set them when w is given."""
        n = self.lpc_info()["nparam"]
        if w is None:
            out = np.zeros(n, dtype=np.float32)
            self.check(self._lib.fs_lpc_weights(self.ctx, out.ctypes.data_as(C.POINTER(C.c_float)), n, 0))
            return out
        w = np.ascontiguousarray(w, dtype=np.float32)
        self.check(self._lib.fs_lpc_weights(self.ctx, w.ctypes.data_as(C.POINTER(C.c_float)), n, 1))

    def lpc_grad(self, feat, tgt, mask):
        """Loss, gradient and predictions of the network for feat [B][h][w][4]."""
        feat = np.ascontiguousarray(feat, dtype=np.float32)
        tgt = np.ascontiguousarray(tgt, dtype=np.float32)
        mask = np.ascontiguousarray(mask, dtype=np.float32)
        n = self.lpc_info()["nparam"]
        g = np.zeros(n, dtype=np.float32)
        pred = np.zeros(tgt.shape, dtype=np.float32)
        loss = C.c_float()
        f = lambda a: a.ctypes.data_as(C.POINTER(C.c_float))
        self.check(self._lib.fs_lpc_grad(self.ctx, f(feat), f(tgt), f(mask), feat.shape[0], f(g),
                                         C.byref(loss), f(pred)))
        return loss.value, g, pred


def batch_run(discharges, steps, t_end=0.0, nthreads=32, check=True, fused=False):
    """Advance independent discharges concurrently in the library (fs_batch_run):
    `steps` main-loop iterations each, or until t >= t_end (nondimensional,
    0 = no limit).  fused: the RK stages of all discharges as one launch per
    stage (fs_batch_run_fused; FP64, DC, no dielectric wall).  Returns (stats
    dicts, return codes); with check, raises if any instance failed."""
    lib = load_library()
    n = len(discharges)
    arr = (C.c_void_p * n)(*[d.ctx for d in discharges])
    st = (abi.FsStats * n)()
    rcs = (C.c_int32 * n)()
    fn = lib.fs_batch_run_fused if fused else lib.fs_batch_run
    rc = fn(arr, n, int(steps), float(t_end), int(nthreads), st, rcs)
    out = [st[i].as_dict() for i in range(n)]
    for d, s in zip(discharges, out):
        d.t, d.dt, d.ts = s["t"], s["dt"], s["steps"]
    if rc != abi.FS_OK and check:
        bad = [i for i in range(n) if rcs[i] != 0]
        raise FluidsimError(rc, "batch: instances %s failed (first: %s)" % (
            bad[:8], discharges[bad[0]].last_error() if bad else ""))
    return out, list(rcs)
