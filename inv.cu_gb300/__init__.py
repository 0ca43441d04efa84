"""Python mirror of inv.cu's solver/filter/misfit/optimizer interface.

A thin ctypes layer over libgbfwi.so (include/gbfwi.h). Class and method
names follow the reference so callers and tests read like the reference's
own code:

    Config        lib/config.h:86-108
    FdmSolver     solver/solver.h:7-268, solver/fdm.h:222-613
    GaussianFilter filter/gaussian.h:37-61
    Misfit        misfit/misfit.h (type 0 waveform, 1 envelope)
    Optimizer     optimizer/optimizer.h (NLCG / L-BFGS by config)

Every computation runs in the CUDA library; there is no CPU path. Importing
works without a GPU (the library loads and its configuration calls work);
solver calls need a CUDA device and raise GbError otherwise.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libgbfwi.so")
GBINV_PATH = os.path.join(HERE, "gbinv")

GB_OK, GB_ERR_ARG, GB_ERR_CUDA, GB_ERR_IO, GB_ERR_BUDGET, GB_ERR_STATE, GB_ERR_MODEL = range(7)
(GB_OUT_X, GB_OUT_Y, GB_OUT_Z, GB_ADSTF_X, GB_ADSTF_Y, GB_ADSTF_Z, GB_LAMBDA, GB_MU, GB_RHO,
 GB_K_LAMBDA, GB_K_MU, GB_K_RHO, GB_STF_X, GB_STF_Y, GB_STF_Z) = range(15)
COMP = {"x": 0, "y": 1, "z": 2}


class GbError(RuntimeError):
    pass


class RequestDesc(ctypes.Structure):
    _fields_ = [("psv", ctypes.c_int), ("nx", ctypes.c_int), ("nz", ctypes.c_int), ("dx", ctypes.c_float),
                ("dz", ctypes.c_float), ("dt", ctypes.c_float), ("nt", ctypes.c_int),
                ("lambda_", ctypes.POINTER(ctypes.c_float)), ("mu", ctypes.POINTER(ctypes.c_float)),
                ("rho", ctypes.POINTER(ctypes.c_float)), ("src", ctypes.c_float * 7), ("nrec", ctypes.c_int),
                ("rec", ctypes.POINTER(ctypes.c_float)), ("obs", ctypes.POINTER(ctypes.c_float)),
                ("abs_width", ctypes.c_int), ("abs_alpha", ctypes.c_float), ("abs_left", ctypes.c_int),
                ("abs_right", ctypes.c_int), ("abs_bottom", ctypes.c_int), ("abs_top", ctypes.c_int),
                ("inv_lambda", ctypes.c_int), ("inv_mu", ctypes.c_int), ("inv_rho", ctypes.c_int),
                ("arrival", ctypes.c_double)]


class ServerStats(ctypes.Structure):
    _fields_ = [("completed", ctypes.c_int), ("wall_s", ctypes.c_double), ("p50_s", ctypes.c_double),
                ("p99_s", ctypes.c_double), ("max_concurrent", ctypes.c_int), ("rounds", ctypes.c_longlong),
                ("launches", ctypes.c_longlong), ("cell_updates", ctypes.c_longlong)]


class GbStats(ctypes.Structure):
    _fields_ = [("forward_ms", ctypes.c_double), ("adjoint_ms", ctypes.c_double),
                ("misfit_ms", ctypes.c_double), ("filter_ms", ctypes.c_double),
                ("step_ms", ctypes.c_double), ("step_launches", ctypes.c_longlong),
                ("launches", ctypes.c_longlong), ("cell_updates", ctypes.c_longlong),
                ("tile_tz", ctypes.c_int), ("tile_tx", ctypes.c_int), ("batch_capacity", ctypes.c_int),
                ("march_bulk", ctypes.c_int), ("cluster_adj", ctypes.c_int), ("cluster_shift", ctypes.c_int)]


_lib = None
_vp = ctypes.c_void_p
_fp = ctypes.POINTER(ctypes.c_float)


def _declare(lib):
    sig = {
        "gb_last_error": (ctypes.c_char_p, []),
        "gb_version": (ctypes.c_int, []),
        "gb_config_load": (_vp, [ctypes.c_char_p, ctypes.c_int, ctypes.POINTER(ctypes.c_char_p)]),
        "gb_config_new": (_vp, [ctypes.c_char_p]),
        "gb_config_free": (None, [_vp]),
        "gb_config_set": (ctypes.c_int, [_vp, ctypes.c_char_p, ctypes.c_char_p]),
        "gb_config_has": (ctypes.c_int, [_vp, ctypes.c_char_p]),
        "gb_config_f": (ctypes.c_float, [_vp, ctypes.c_char_p]),
        "gb_config_i": (ctypes.c_int, [_vp, ctypes.c_char_p]),
        "gb_config_path": (ctypes.c_char_p, [_vp]),
        "gb_config_nsrc": (ctypes.c_int, [_vp]),
        "gb_config_nrec": (ctypes.c_int, [_vp]),
        "gb_config_source": (ctypes.c_int, [_vp, ctypes.c_int, _fp]),
        "gb_config_station": (ctypes.c_int, [_vp, ctypes.c_int, _fp]),
        "gb_config_add_source": (ctypes.c_int, [_vp, _fp]),
        "gb_config_add_station": (ctypes.c_int, [_vp, _fp]),
        "gb_solver_create": (_vp, [_vp]),
        "gb_solver_create_grid": (_vp, [_vp, ctypes.c_int, ctypes.c_int, ctypes.c_float, ctypes.c_float]),
        "gb_solver_destroy": (None, [_vp]),
        "gb_import_model": (ctypes.c_int, [_vp, ctypes.c_int]),
        "gb_set_model_points": (ctypes.c_int, [_vp, ctypes.c_int, _fp, _fp, _fp, _fp, _fp]),
        "gb_set_model_grid": (ctypes.c_int, [_vp, _fp, _fp, _fp]),
        "gb_run_forward": (ctypes.c_int, [_vp, ctypes.c_int, ctypes.c_int, ctypes.c_int]),
        "gb_run_adjoint": (ctypes.c_int, [_vp, ctypes.c_int, ctypes.c_int]),
        "gb_init_kernels": (ctypes.c_int, [_vp]),
        "gb_export_axis": (ctypes.c_int, [_vp]),
        "gb_export_model": (ctypes.c_int, [_vp, ctypes.c_int]),
        "gb_export_kernel": (ctypes.c_int, [_vp, ctypes.c_int]),
        "gb_export_traces": (ctypes.c_int, [_vp, ctypes.c_int]),
        "gb_infer_grid": (ctypes.c_int, [ctypes.c_char_p, ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_int),
                                         ctypes.POINTER(ctypes.c_float), ctypes.POINTER(ctypes.c_float),
                                         ctypes.POINTER(ctypes.c_int)]),
        "gb_su_write": (ctypes.c_int, [ctypes.c_char_p, _vp, ctypes.c_int, ctypes.c_int, ctypes.c_float,
                                       ctypes.c_float, ctypes.c_float, _vp, _vp]),
        "gb_su_read": (ctypes.c_int, [ctypes.c_char_p, _vp, ctypes.c_int, ctypes.c_int]),
        "gb_solver_ptr": (_vp, [_vp, ctypes.c_int]),
        "gb_solver_dims": (ctypes.c_int, [_vp] + [ctypes.POINTER(ctypes.c_int)] * 5),
        "gb_solver_steps": (ctypes.c_int, [_vp] + [_fp] * 3),
        "gb_run_forward_batch": (ctypes.c_int, [_vp, ctypes.POINTER(ctypes.c_int), ctypes.c_int]),
        "gb_run_adjoint_batch": (ctypes.c_int, [_vp, ctypes.POINTER(ctypes.c_int), ctypes.c_int]),
        "gb_slot_ptr": (_vp, [_vp, ctypes.c_int, ctypes.c_int]),
        "gb_solver_batch_capacity": (ctypes.c_int, [_vp]),
        "gb_solver_set_option": (ctypes.c_int, [_vp, ctypes.c_char_p, ctypes.c_double]),
        "gb_solver_stats": (ctypes.c_int, [_vp, ctypes.POINTER(GbStats), ctypes.c_int]),
        "gb_filter_create": (_vp, [ctypes.c_int, ctypes.c_int, ctypes.c_int]),
        "gb_filter_apply": (ctypes.c_int, [_vp, _vp]),
        "gb_filter_destroy": (None, [_vp]),
        "gb_filter_apply_noalloc": (ctypes.c_int, [ctypes.c_int, ctypes.c_int, ctypes.c_int, _vp]),
        "gb_misfit_create": (_vp, [_vp, _vp, _vp]),
        "gb_misfit_create_obs": (_vp, [ctypes.c_int, _vp, _vp, _fp, _fp, _fp]),
        "gb_misfit_set_obs": (ctypes.c_int, [_vp, _fp, _fp, _fp]),
        "gb_misfit_set_obs_async": (ctypes.c_int, [_vp, _fp, _fp, _fp]),
        "gb_misfit_run": (ctypes.c_int, [_vp, ctypes.c_int, ctypes.c_int, ctypes.POINTER(ctypes.c_double)]),
        "gb_misfit_trace_values": (ctypes.c_int, [_vp, ctypes.POINTER(ctypes.c_double), ctypes.c_size_t]),
        "gb_misfit_destroy": (None, [_vp]),
        "gb_optimizer_create": (_vp, [_vp, _vp, _vp]),
        "gb_optimizer_run": (ctypes.c_int, [_vp]),
        "gb_optimizer_history": (ctypes.c_int, [_vp, ctypes.POINTER(ctypes.c_double), ctypes.c_int]),
        "gb_optimizer_evaluations": (ctypes.c_int, [_vp, ctypes.POINTER(ctypes.c_double), ctypes.c_int]),
        "gb_linesearch_step": (ctypes.c_double, [ctypes.c_int, _vp, _vp, ctypes.c_int, _vp, _vp, ctypes.c_int,
                                                 ctypes.c_int, ctypes.c_int, ctypes.c_double, ctypes.c_double,
                                                 ctypes.POINTER(ctypes.c_int)]),
        "gb_optimizer_destroy": (None, [_vp]),
        "gb_dot64": (ctypes.c_int, [_vp, _vp, ctypes.c_size_t, ctypes.POINTER(ctypes.c_double)]),
        "gb_amax64": (ctypes.c_int, [_vp, ctypes.c_size_t, ctypes.POINTER(ctypes.c_double)]),
        "gb_device_malloc": (_vp, [ctypes.c_size_t]),
        "gb_device_free": (ctypes.c_int, [_vp]),
        "gb_memcpy_d2h": (ctypes.c_int, [_vp, _vp, ctypes.c_size_t]),
        "gb_memcpy_h2d": (ctypes.c_int, [_vp, _vp, ctypes.c_size_t]),
        "gb_device_sync": (ctypes.c_int, []),
        "gb_device_count": (ctypes.c_int, []),
        "gb_host_malloc": (_vp, [ctypes.c_size_t]),
        "gb_host_free": (ctypes.c_int, [_vp]),
        "gb_device_select": (ctypes.c_int, [ctypes.c_int]),
        "gb_solver_timer": (ctypes.c_int, [_vp, ctypes.c_int, ctypes.POINTER(ctypes.c_double)]),
        "gb_server_create": (_vp, [ctypes.c_int, ctypes.c_int, ctypes.c_double, ctypes.c_int]),
        "gb_server_set_option": (ctypes.c_int, [_vp, ctypes.c_char_p, ctypes.c_double]),
        "gb_server_submit": (ctypes.c_longlong, [_vp, ctypes.POINTER(RequestDesc)]),
        "gb_server_run": (ctypes.c_int, [_vp]),
        "gb_server_result": (ctypes.c_int, [_vp, ctypes.c_longlong, _fp, _fp, _fp, ctypes.POINTER(ctypes.c_double),
                                            ctypes.POINTER(ctypes.c_double)]),
        "gb_server_report": (ctypes.c_int, [_vp, ctypes.POINTER(ServerStats)]),
        "gb_server_destroy": (None, [_vp]),
    }
    for name, (res, args) in sig.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    return lib


def lib():
    """The loaded libgbfwi.so; raises if it was not built (no fallback)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise GbError("libgbfwi.so is not built: run `python -c \"import __graft_entry__ as g; g.build()\"`")
        _lib = _declare(ctypes.CDLL(LIB_PATH))
    return _lib


def last_error() -> str:
    return lib().gb_last_error().decode(errors="replace")


def check(rc: int, what: str = "") -> None:
    if rc != GB_OK:
        raise GbError("%s failed (%d): %s" % (what or "gbfwi call", rc, last_error()))


def device_count() -> int:
    return lib().gb_device_count()


def _f32(a):
    return np.ascontiguousarray(a, dtype=np.float32)


def _ptr(a):
    return a.ctypes.data_as(_fp) if a is not None else None


def d2h(dptr, n, dtype=np.float32) -> np.ndarray:
    out = np.empty(n, dtype=dtype)
    if n:
        check(lib().gb_memcpy_d2h(out.ctypes.data_as(_vp), dptr, out.nbytes), "gb_memcpy_d2h")
    return out


def h2d(dptr, arr) -> None:
    arr = np.ascontiguousarray(arr)
    if arr.size:
        check(lib().gb_memcpy_h2d(dptr, arr.ctypes.data_as(_vp), arr.nbytes), "gb_memcpy_h2d")


class PinnedArray:
    """A float32 numpy view of pinned host memory from the library."""

    def __init__(self, n):
        self.n = int(n)
        self.ptr = lib().gb_host_malloc(max(1, self.n * 4))
        if not self.ptr:
            raise GbError(last_error())
        buf = (ctypes.c_float * max(1, self.n)).from_address(self.ptr)
        self.array = np.ctypeslib.as_array(buf)[: self.n]

    def __del__(self):
        if getattr(self, "ptr", None) and _lib is not None:
            self.array = None
            _lib.gb_host_free(self.ptr)
            self.ptr = None


def select_device(dev: int) -> None:
    check(lib().gb_device_select(int(dev)), "gb_device_select")


class DeviceArray:
    """A float32 device buffer owned by the library's allocator."""

    def __init__(self, host):
        host = _f32(host)
        self.n = host.size
        self.ptr = lib().gb_device_malloc(max(1, host.nbytes))
        if not self.ptr:
            raise GbError(last_error())
        h2d(self.ptr, host)

    def numpy(self):
        return d2h(self.ptr, self.n)

    def __del__(self):
        if getattr(self, "ptr", None) and _lib is not None:
            _lib.gb_device_free(self.ptr)
            self.ptr = None


# ----------------------------------------------------------------------------
class Config:
    """Config (lib/config.h:86-108)."""

    def __init__(self, handle):
        self._h = handle

    @classmethod
    def load(cls, directory: str, overrides: dict | None = None):
        ov = ["-%s=%s" % (k, v) for k, v in (overrides or {}).items()]
        arr = (ctypes.c_char_p * max(1, len(ov)))(*[s.encode() for s in ov])
        h = lib().gb_config_load(directory.encode(), len(ov), arr)
        if not h:
            raise GbError(last_error())
        return cls(h)

    @classmethod
    def new(cls, directory: str = ".", values: dict | None = None, sources=(), stations=()):
        h = lib().gb_config_new(directory.encode())
        c = cls(h)
        for k, v in (values or {}).items():
            c.set(k, v)
        for s in sources:
            check(lib().gb_config_add_source(h, _ptr(_f32(s))), "add_source")
        for r in stations:
            check(lib().gb_config_add_station(h, _ptr(_f32(r))), "add_station")
        return c

    def set(self, key, value):
        check(lib().gb_config_set(self._h, key.encode(), str(value).encode()), "config set")

    def f(self, key) -> float:
        return float(lib().gb_config_f(self._h, key.encode()))

    def i(self, key) -> int:
        return int(lib().gb_config_i(self._h, key.encode()))

    def has(self, key) -> bool:
        return bool(lib().gb_config_has(self._h, key.encode()))

    @property
    def path(self) -> str:
        return lib().gb_config_path(self._h).decode()

    @property
    def src(self):
        out = []
        buf = np.zeros(7, np.float32)
        for s in range(lib().gb_config_nsrc(self._h)):
            check(lib().gb_config_source(self._h, s, _ptr(buf)))
            out.append(buf.tolist())
        return out

    @property
    def rec(self):
        out = []
        buf = np.zeros(2, np.float32)
        for r in range(lib().gb_config_nrec(self._h)):
            check(lib().gb_config_station(self._h, r, _ptr(buf)))
            out.append(buf.tolist())
        return out

    def __del__(self):
        if getattr(self, "_h", None) and _lib is not None:
            _lib.gb_config_free(self._h)
            self._h = None


class FdmSolver:
    """FdmSolver (solver/fdm.h:222-613) behind the C ABI."""

    def __init__(self, config: Config, grid=None):
        self.config = config
        if grid is None:
            h = lib().gb_solver_create(config._h)
        else:
            nx, nz, xmax, zmax = grid
            h = lib().gb_solver_create_grid(config._h, int(nx), int(nz), float(xmax), float(zmax))
        if not h:
            raise GbError(last_error())
        self._h = h
        d = [ctypes.c_int() for _ in range(5)]
        check(lib().gb_solver_dims(h, *[ctypes.byref(x) for x in d]))
        self.nx, self.nz, self.nt, self.nsrc, self.nrec = [x.value for x in d]
        f = [ctypes.c_float() for _ in range(3)]
        check(lib().gb_solver_steps(h, *[ctypes.byref(x) for x in f]))
        self.dx, self.dz, self.dt = [x.value for x in f]

    # -- reference methods
    def importModel(self, model: bool):
        check(lib().gb_import_model(self._h, int(bool(model))), "importModel")

    def runForward(self, isrc: int, trace: bool = False, snapshot: bool = False):
        check(lib().gb_run_forward(self._h, int(isrc), int(trace), int(snapshot)), "runForward")

    def runAdjoint(self, isrc: int, snapshot: bool = False):
        check(lib().gb_run_adjoint(self._h, int(isrc), int(snapshot)), "runAdjoint")

    def initKernels(self):
        check(lib().gb_init_kernels(self._h), "initKernels")

    def exportAxis(self):
        check(lib().gb_export_axis(self._h), "exportAxis")

    def exportModel(self, n: int = 0):
        check(lib().gb_export_model(self._h, n), "exportModel")

    def exportKernel(self, n: int = 0):
        check(lib().gb_export_kernel(self._h, n), "exportKernel")

    def exportTraces(self, isrc: int):
        check(lib().gb_export_traces(self._h, isrc), "exportTraces")

    # -- model intake
    def set_model_points(self, x, z, a, b, rho):
        arrs = [_f32(v) for v in (x, z, a, b, rho)]
        check(lib().gb_set_model_points(self._h, arrs[0].size, *[_ptr(v) for v in arrs]), "set_model_points")

    def set_model_grid(self, lam, mu, rho):
        arrs = [_f32(v).ravel() for v in (lam, mu, rho)]
        if any(a.size != self.nx * self.nz for a in arrs):
            raise GbError("model arrays must have nx*nz elements")
        check(lib().gb_set_model_grid(self._h, *[_ptr(v) for v in arrs]), "set_model_grid")

    # -- buffers
    def ptr(self, which: int):
        return lib().gb_solver_ptr(self._h, which)

    def grid_array(self, which: int) -> np.ndarray:
        p = self.ptr(which)
        if not p:
            raise GbError("buffer %d is not allocated" % which)
        return d2h(p, self.nx * self.nz)

    def model(self):
        return {k: self.grid_array(w) for k, w in (("lambda", GB_LAMBDA), ("mu", GB_MU), ("rho", GB_RHO))}

    def kernels(self):
        return {k: self.grid_array(w) for k, w in
                (("k_lambda", GB_K_LAMBDA), ("k_mu", GB_K_MU), ("k_rho", GB_K_RHO))}

    def out(self, comp: str, slot: int = 0) -> np.ndarray:
        p = lib().gb_slot_ptr(self._h, slot, GB_OUT_X + COMP[comp])
        if not p:
            raise GbError("no traces for component %s" % comp)
        return d2h(p, self.nrec * self.nt).reshape(self.nrec, self.nt)

    def set_adstf(self, comp: str, data, slot: int = 0):
        p = lib().gb_slot_ptr(self._h, slot, GB_ADSTF_X + COMP[comp])
        if not p:
            raise GbError("no adjoint source for component %s" % comp)
        h2d(p, _f32(data).ravel())

    def adstf(self, comp: str, slot: int = 0) -> np.ndarray:
        p = lib().gb_slot_ptr(self._h, slot, GB_ADSTF_X + COMP[comp])
        return d2h(p, self.nrec * self.nt).reshape(self.nrec, self.nt)

    # -- batched extension
    def run_forward_batch(self, shots):
        arr = (ctypes.c_int * len(shots))(*shots)
        check(lib().gb_run_forward_batch(self._h, arr, len(shots)), "run_forward_batch")

    def run_adjoint_batch(self, shots):
        arr = (ctypes.c_int * len(shots))(*shots)
        check(lib().gb_run_adjoint_batch(self._h, arr, len(shots)), "run_adjoint_batch")

    @property
    def capacity(self) -> int:
        return lib().gb_solver_batch_capacity(self._h)

    def set_option(self, key: str, value):
        check(lib().gb_solver_set_option(self._h, key.encode(), float(value)), "set_option " + key)

    def timer_begin(self):
        check(lib().gb_solver_timer(self._h, 1, None), "timer begin")

    def timer_end(self) -> float:
        v = ctypes.c_double()
        check(lib().gb_solver_timer(self._h, 0, ctypes.byref(v)), "timer end")
        return v.value

    def stats(self, reset: bool = False) -> GbStats:
        s = GbStats()
        check(lib().gb_solver_stats(self._h, ctypes.byref(s), int(reset)))
        return s

    def close(self):
        if getattr(self, "_h", None) and _lib is not None:
            _lib.gb_solver_destroy(self._h)
            self._h = None

    def __del__(self):
        self.close()


class GaussianFilter:
    """GaussianFilter (filter/gaussian.h:37-61)."""

    def __init__(self, nx: int, nz: int, sigma: int):
        self._h = lib().gb_filter_create(nx, nz, sigma)
        if not self._h:
            raise GbError(last_error())
        self.nx, self.nz = nx, nz

    def apply(self, dptr):
        check(lib().gb_filter_apply(self._h, dptr), "filter apply")

    def apply_host(self, data) -> np.ndarray:
        d = DeviceArray(_f32(data).ravel())
        self.apply(d.ptr)
        return d.numpy()

    def close(self):
        if getattr(self, "_h", None) and _lib is not None:
            _lib.gb_filter_destroy(self._h)
            self._h = None

    def __del__(self):
        self.close()


class Misfit:
    """Misfit (misfit/misfit.h) — waveform (0) or envelope (1)."""

    def __init__(self, handle, solver, filt=None):
        self._h = handle
        self.solver = solver
        self.filter = filt

    @classmethod
    def from_config(cls, config: Config, solver: FdmSolver, filt: GaussianFilter | None = None):
        h = lib().gb_misfit_create(config._h, solver._h, filt._h if filt else None)
        if not h:
            raise GbError(last_error())
        return cls(h, solver, filt)

    @classmethod
    def from_obs(cls, kind: int, solver: FdmSolver, obs: dict, filt: GaussianFilter | None = None):
        arr = {c: (_f32(obs[c]).ravel() if obs.get(c) is not None else None) for c in "xyz"}
        h = lib().gb_misfit_create_obs(kind, solver._h, filt._h if filt else None,
                                       *[_ptr(arr[c]) for c in "xyz"])
        if not h:
            raise GbError(last_error())
        return cls(h, solver, filt)

    def set_obs(self, obs: dict):
        arr = {c: (_f32(obs[c]).ravel() if obs.get(c) is not None else None) for c in "xyz"}
        check(lib().gb_misfit_set_obs(self._h, *[_ptr(arr[c]) for c in "xyz"]), "set_obs")

    def set_obs_async(self, obs: dict):
        """gb_misfit_set_obs_async: the copies overlap the next run's forward
        pass; the arrays are kept alive here until that run returns."""
        arr = {c: (_f32(obs[c]).ravel() if obs.get(c) is not None else None) for c in "xyz"}
        check(lib().gb_misfit_set_obs_async(self._h, *[_ptr(arr[c]) for c in "xyz"]), "set_obs_async")
        self._obs_hold = arr

    def run(self, kernel: bool = False, snapshot: bool = False) -> float:
        v = ctypes.c_double()
        check(lib().gb_misfit_run(self._h, int(kernel), int(snapshot), ctypes.byref(v)), "misfit run")
        self._obs_hold = None
        return v.value

    def trace_values(self) -> np.ndarray:
        ncomp = (1 if self.solver.config.i("sh") else 0) + (2 if self.solver.config.i("psv") else 0)
        n = self.solver.nsrc * self.solver.nrec * ncomp
        out = np.zeros(n, np.float64)
        check(lib().gb_misfit_trace_values(self._h, out.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), n))
        return out

    def close(self):
        if getattr(self, "_h", None) and _lib is not None:
            _lib.gb_misfit_destroy(self._h)
            self._h = None

    def __del__(self):
        self.close()


def infer_grid(directory: str):
    """(nx, nz, xmax, zmax, npt) of <directory>/model_true, as FdmSolver::init
    infers them (solver/fdm.h:354-391)."""
    nx, nz, npt = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
    xm, zm = ctypes.c_float(), ctypes.c_float()
    check(lib().gb_infer_grid(directory.encode(), ctypes.byref(nx), ctypes.byref(nz), ctypes.byref(xm),
                              ctypes.byref(zm), ctypes.byref(npt)), "infer_grid")
    return nx.value, nz.value, xm.value, zm.value, npt.value


def su_write(path: str, traces, dt: float, xs: float, zs: float, rec_x, rec_z) -> None:
    """An SU file as Solver::exportTraces writes it (solver/solver.h:38-108);
    traces [nrec, nt] in host memory."""
    t = np.ascontiguousarray(traces, dtype=np.float32)
    rx, rz = _f32(rec_x), _f32(rec_z)
    nrec, nt = t.shape
    check(lib().gb_su_write(path.encode(), t.ctypes.data_as(_vp), nrec, nt, float(dt), float(xs), float(zs),
                            rx.ctypes.data_as(_vp), rz.ctypes.data_as(_vp)), "su_write")


def su_read(path: str, nrec: int, nt: int) -> np.ndarray:
    """Traces [nrec, nt] of an SU file as Misfit::importTraces reads them."""
    out = np.zeros((nrec, nt), np.float32)
    check(lib().gb_su_read(path.encode(), out.ctypes.data_as(_vp), nrec, nt), "su_read")
    return out


def linesearch_step(optimizer: int, lens, vals, gtg, gtp, step_count: int, ls_step: int, ls_thresh: float,
                    step_max: float):
    """The line-search step rule of the optimizer (bracket for NLCG,
    backtrack for L-BFGS, optimizer/optimizer.h:267-357) on a history, on the
    host: returns (step, status)."""
    d = lambda a: np.ascontiguousarray(a, dtype=np.float64)
    lens, vals, gtg, gtp = d(lens), d(vals), d(gtg), d(gtp)
    st = ctypes.c_int(-2)
    a = lib().gb_linesearch_step(int(optimizer), lens.ctypes.data_as(_vp), vals.ctypes.data_as(_vp), int(lens.size),
                                 gtg.ctypes.data_as(_vp), gtp.ctypes.data_as(_vp), int(gtg.size), int(step_count),
                                 int(ls_step), float(ls_thresh), float(step_max), ctypes.byref(st))
    if st.value == -2:
        raise GbError("linesearch_step: " + last_error())
    return a, st.value


class Optimizer:
    """Optimizer (optimizer/optimizer.h): NLCG or L-BFGS from `optimizer`."""

    def __init__(self, config: Config, solver: FdmSolver, misfit: Misfit):
        self._h = lib().gb_optimizer_create(config._h, solver._h, misfit._h)
        if not self._h:
            raise GbError(last_error())
        self.misfit = misfit

    def run(self):
        check(lib().gb_optimizer_run(self._h), "optimizer run")

    def history(self) -> np.ndarray:
        n = lib().gb_optimizer_history(self._h, None, 0)
        out = np.zeros(max(n, 1), np.float64)
        lib().gb_optimizer_history(self._h, out.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), n)
        return out[:n]

    def evaluations(self) -> np.ndarray:
        """[n, 3]: (kind, alpha, value) of every misfit evaluation of the
        last run (kind 1 gradient, 0 line-search step, 2 final)."""
        n = lib().gb_optimizer_evaluations(self._h, None, 0)
        out = np.zeros(max(3 * n, 3), np.float64)
        lib().gb_optimizer_evaluations(self._h, out.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), n)
        return out[:3 * n].reshape(n, 3)

    def close(self):
        if getattr(self, "_h", None) and _lib is not None:
            _lib.gb_optimizer_destroy(self._h)
            self._h = None

    def __del__(self):
        self.close()


class Server:
    """Continuous-batching engine for forward+adjoint shot requests."""

    def __init__(self, sfe=10, ckpt=0, hbm_budget_gb=0.0, max_slots=0):
        self._h = lib().gb_server_create(int(sfe), int(ckpt), float(hbm_budget_gb), int(max_slots))
        if not self._h:
            raise GbError(last_error())
        self._keep = {}

    def set_option(self, key, value):
        """Engine option set before run(): "tile" (step kernel configuration 1..20), "tma" (0/1), "streams" (1/2)."""
        check(lib().gb_server_set_option(self._h, key.encode(), float(value)))

    def submit(self, *, psv, nx, nz, dx, dt, nt, lam, mu, rho, src, rec, obs=None, arrival=0.0, abs_width=20,
               abs_alpha=0.015, abs_edges=(1, 1, 1, 0), inv=(1, 1, 1), dz=None) -> int:
        arrs = [_f32(a).ravel() for a in (lam, mu, rho)]
        recs = _f32(rec).ravel()
        ob = _f32(obs).ravel() if obs is not None else None
        d = RequestDesc()
        d.psv, d.nx, d.nz, d.dx, d.dz, d.dt, d.nt = int(psv), nx, nz, dx, dz if dz else dx, dt, nt
        d.lambda_, d.mu, d.rho = (_ptr(a) for a in arrs)
        d.src = (ctypes.c_float * 7)(*src)
        d.nrec = recs.size // 2
        d.rec = _ptr(recs)
        d.obs = _ptr(ob) if ob is not None else None
        d.abs_width, d.abs_alpha = abs_width, abs_alpha
        d.abs_left, d.abs_right, d.abs_bottom, d.abs_top = abs_edges
        d.inv_lambda, d.inv_mu, d.inv_rho = inv
        d.arrival = arrival
        rid = lib().gb_server_submit(self._h, ctypes.byref(d))
        if rid < 0:
            raise GbError(last_error())
        self._keep[rid] = (arrs, recs, ob, nx * nz)
        return rid

    def run(self):
        check(lib().gb_server_run(self._h), "server run")

    def result(self, rid):
        n = self._keep[rid][3]
        ks = [np.zeros(n, np.float32) for _ in range(3)]
        mis, lat = ctypes.c_double(), ctypes.c_double()
        check(lib().gb_server_result(self._h, rid, *[_ptr(k) for k in ks], ctypes.byref(mis), ctypes.byref(lat)),
              "server result")
        return {"k_lambda": ks[0], "k_mu": ks[1], "k_rho": ks[2], "misfit": mis.value, "latency": lat.value}

    def stats(self) -> ServerStats:
        s = ServerStats()
        check(lib().gb_server_report(self._h, ctypes.byref(s)))
        return s

    def close(self):
        if getattr(self, "_h", None) and _lib is not None:
            _lib.gb_server_destroy(self._h)
            self._h = None

    def __del__(self):
        self.close()


def dot64(pa, pb, n) -> float:
    v = ctypes.c_double()
    check(lib().gb_dot64(pa, pb, n, ctypes.byref(v)), "gb_dot64")
    return v.value


def amax64(pa, n) -> float:
    v = ctypes.c_double()
    check(lib().gb_amax64(pa, n, ctypes.byref(v)), "gb_amax64")
    return v.value
