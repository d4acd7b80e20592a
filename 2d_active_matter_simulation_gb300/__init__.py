"""Python front end of libactflow (the GB300 solver behind include/actflow.h).

The package is a thin ctypes binding over the C ABI: no computation happens in
Python.  Importing it loads ``lib/libactflow.so`` (built in-tree by
``build.py``); if the library is missing the import raises, so a test or
benchmark can never run on a silent fallback.

    import importlib
    am = importlib.import_module("2d_active_matter_simulation_gb300")
    sim = am.Solver(nx=256, ny=256, lx=..., ly=..., dt=..., lam=..., alpha=..., beta=...)
    sim.set_state(w_hat, mean)          # [ny][nx//2+1] complex, mean[2]
    energy = sim.step(100)              # energy of the state entering each step
    w_hat, mean = sim.get_state()
"""
import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "lib", "libactflow.so")
CLI_PATH = os.path.join(HERE, "lib", "actflow")

(AM_OK, AM_ERR_ARG, AM_ERR_CUDA, AM_ERR_NAN, AM_ERR_IO, AM_ERR_SPEC, AM_ERR_OOM, AM_ERR_UNSUPPORTED,
 AM_ERR_TIMEOUT) = range(9)
ORDER = {"arrival": 0, "shortest": 1}
FP32, FP64, DF64 = 0, 1, 2   # am_precision; DF64: double-float (two floats per real)
PRECISIONS = {"fp32": FP32, "fp64": FP64, "df64": DF64}


def _prec(precision):
    """am_precision of a name ("fp32", "fp64", "df64") or of the enum value."""
    if precision in PRECISIONS:
        return PRECISIONS[precision]
    if precision in (FP32, FP64, DF64):
        return int(precision)
    raise ValueError(f"unknown precision {precision!r}")
DEALIAS = {"reference": 0, "half": 1, "none": 2}
# integrating factors: per value in the state precision (lin_func) or precomputed in double
IF_FACTORS = {"auto": 0, "float": 1, "double": 2}
FORM_REFERENCE, FORM_GENERAL = 0, 1


class Params(ctypes.Structure):
    _fields_ = [
        ("nx", ctypes.c_int), ("ny", ctypes.c_int),
        ("lx", ctypes.c_double), ("ly", ctypes.c_double), ("dt", ctypes.c_double),
        ("lam", ctypes.c_double), ("alpha", ctypes.c_double), ("beta", ctypes.c_double),
        ("gamma0", ctypes.c_double), ("gamma2", ctypes.c_double),
        ("form", ctypes.c_int), ("dealias", ctypes.c_int), ("precision", ctypes.c_int),
        ("if_factors", ctypes.c_int), ("reserved", ctypes.c_int * 4),
    ]


class Spec(ctypes.Structure):
    _fields_ = [
        ("T", ctypes.c_double), ("dt", ctypes.c_double), ("lx", ctypes.c_double), ("ly", ctypes.c_double),
        ("nx", ctypes.c_int), ("ny", ctypes.c_int),
        ("lam", ctypes.c_double), ("alpha", ctypes.c_double), ("beta", ctypes.c_double),
        ("dt_snap", ctypes.c_double), ("gamma0", ctypes.c_double), ("gamma2", ctypes.c_double),
        ("has_gamma", ctypes.c_int), ("precision", ctypes.c_int), ("dealias", ctypes.c_int),
        ("initial", ctypes.c_char * 256), ("directory", ctypes.c_char * 1024),
    ]


class ServerConfig(ctypes.Structure):
    _fields_ = [("hbm_budget_bytes", ctypes.c_longlong), ("max_active", ctypes.c_int),
                ("chunk_steps", ctypes.c_int), ("order", ctypes.c_int), ("max_active_fp64", ctypes.c_int),
                ("reserved", ctypes.c_int * 4)]


class Job(ctypes.Structure):
    _fields_ = [("params", Params), ("nsteps", ctypes.c_longlong), ("w_hat", ctypes.c_void_p),
                ("mean", ctypes.c_double * 2), ("seed", ctypes.c_ulonglong), ("kmin", ctypes.c_double),
                ("kmax", ctypes.c_double), ("rms", ctypes.c_double), ("want_state", ctypes.c_int),
                ("want_energy", ctypes.c_int), ("reserved", ctypes.c_int * 4)]


class JobResult(ctypes.Structure):
    _fields_ = [("id", ctypes.c_longlong), ("status", ctypes.c_int), ("t_submit", ctypes.c_double),
                ("t_admit", ctypes.c_double), ("t_done", ctypes.c_double), ("mean", ctypes.c_double * 2),
                ("steps_done", ctypes.c_longlong), ("error", ctypes.c_char * 256)]


class ServerInfo(ctypes.Structure):
    _fields_ = [("elapsed_s", ctypes.c_double), ("jobs_submitted", ctypes.c_longlong),
                ("jobs_done", ctypes.c_longlong), ("jobs_pending", ctypes.c_longlong),
                ("jobs_active", ctypes.c_int), ("peak_active", ctypes.c_int),
                ("grid_point_steps", ctypes.c_longlong), ("device_bytes_reserved", ctypes.c_longlong),
                ("peak_device_bytes", ctypes.c_longlong)]


class ActflowError(RuntimeError):
    def __init__(self, status, msg):
        super().__init__(msg)
        self.status = status


def _load():
    if not os.path.exists(LIB_PATH):
        raise ImportError(
            f"libactflow.so not found at {LIB_PATH}: build it first "
            "(python -c 'import __graft_entry__ as g; g.build()')")
    L = ctypes.CDLL(LIB_PATH)
    vp, dp, ip = ctypes.c_void_p, ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_int)
    hp = ctypes.c_void_p
    sig = {
        "am_create": ([ctypes.POINTER(Params), ctypes.POINTER(hp)], ctypes.c_int),
        "am_destroy": ([hp], ctypes.c_int),
        "am_set_stream": ([hp, vp], ctypes.c_int),
        "am_set_state": ([hp, vp, dp], ctypes.c_int),
        "am_set_state_real": ([hp, vp, dp, ctypes.c_int], ctypes.c_int),
        "am_get_state": ([hp, vp, dp], ctypes.c_int),
        "am_step": ([hp, ctypes.c_int, dp, ip], ctypes.c_int),
        "am_step_async": ([hp, ctypes.c_int], ctypes.c_int),
        "am_sync": ([hp], ctypes.c_int),
        "am_step_profiled": ([hp, ctypes.c_int, dp, dp], ctypes.c_int),
        "am_row_passes_async": ([hp, ctypes.c_int], ctypes.c_int),
        "am_step_noalloc": ([ctypes.POINTER(Params), vp, vp, ctypes.c_int, vp, vp], ctypes.c_int),
        "am_launches_per_step": ([hp], ctypes.c_int),
        "am_device_bytes": ([hp], ctypes.c_longlong),
        "am_kx_carried": ([hp], ctypes.c_int),
        "am_status_string": ([ctypes.c_int], ctypes.c_char_p),
        "am_last_error": ([hp], ctypes.c_char_p),
        "am_mask_value": ([ctypes.c_int] * 5, ctypes.c_int),
        "am_ic_bandlimited": ([ctypes.c_int, ctypes.c_int, ctypes.c_ulonglong, ctypes.c_double,
                               ctypes.c_double, ctypes.c_double, dp], ctypes.c_int),
        "am_spec_read": ([ctypes.c_char_p, ctypes.POINTER(Spec), ctypes.c_char_p, ctypes.c_int], ctypes.c_int),
        "am_write_snapshot": ([ctypes.c_char_p, ctypes.c_int, ctypes.c_int, ctypes.c_int, vp, dp], ctypes.c_int),
        "am_read_snapshot": ([ctypes.c_char_p, ctypes.c_int, ctypes.c_int, ctypes.c_int, vp, dp], ctypes.c_int),
        "am_append_energy": ([ctypes.c_char_p, ctypes.c_longlong, ctypes.c_int, ctypes.c_float, dp,
                              ctypes.c_int], ctypes.c_int),
        "am_cli_main": ([ctypes.c_int, ctypes.POINTER(ctypes.c_char_p)], ctypes.c_int),
        "am_batch_create": ([ctypes.POINTER(Params), ctypes.c_int, ctypes.POINTER(hp)], ctypes.c_int),
        "am_batch_destroy": ([hp], ctypes.c_int),
        "am_batch_set_state": ([hp, ctypes.c_int, vp, dp], ctypes.c_int),
        "am_batch_get_state": ([hp, ctypes.c_int, vp, dp], ctypes.c_int),
        "am_batch_step": ([hp, ctypes.c_int, dp, ip], ctypes.c_int),
        "am_batch_last_error": ([hp], ctypes.c_char_p),
        "am_ragged_create": ([ctypes.POINTER(Params), ctypes.POINTER(ctypes.c_longlong), ctypes.c_int,
                              ctypes.POINTER(hp)], ctypes.c_int),
        "am_ragged_destroy": ([hp], ctypes.c_int),
        "am_ragged_set_state": ([hp, ctypes.c_int, vp, dp], ctypes.c_int),
        "am_ragged_get_state": ([hp, ctypes.c_int, vp, dp], ctypes.c_int),
        "am_ragged_run": ([hp, ctypes.POINTER(dp), ip, ctypes.POINTER(ctypes.c_longlong)], ctypes.c_int),
        "am_ragged_device_bytes": ([hp], ctypes.c_longlong),
        "am_ragged_classes": ([hp], ctypes.c_int),
        "am_ragged_set_mode": ([hp, ctypes.c_int], ctypes.c_int),
        "am_ragged_last_error": ([hp], ctypes.c_char_p),
        "am_server_create": ([ctypes.POINTER(ServerConfig), ctypes.POINTER(hp)], ctypes.c_int),
        "am_server_submit": ([hp, ctypes.POINTER(Job), ctypes.POINTER(ctypes.c_longlong)], ctypes.c_int),
        "am_server_wait": ([hp, ctypes.c_longlong, ctypes.c_double, ctypes.POINTER(JobResult), vp, dp],
                           ctypes.c_int),
        "am_server_stats": ([hp, ctypes.POINTER(ServerInfo)], ctypes.c_int),
        "am_server_destroy": ([hp], ctypes.c_int),
        "am_footprint_bytes": ([ctypes.POINTER(Params)], ctypes.c_longlong),
        "am_set_column_shape": ([ctypes.c_int, ctypes.c_int, ctypes.c_int], ctypes.c_int),
        "am_column_shape": ([ctypes.c_int, ctypes.c_int], ctypes.c_int),
        "am_autotune": ([ctypes.POINTER(Params), ctypes.c_int, dp, dp], ctypes.c_int),
        "am_set_row_shape": ([ctypes.c_int, ctypes.c_int, ctypes.c_int], ctypes.c_int),
        "am_row_shape": ([ctypes.c_int, ctypes.c_int], ctypes.c_int),
    }
    for name, (args, res) in sig.items():
        f = getattr(L, name)
        f.argtypes = args
        f.restype = res
    return L


lib = _load()

# Every symbol include/actflow.h declares (checked by the CPU test suite).
EXPORTED = [
    "am_create", "am_destroy", "am_set_stream", "am_set_state", "am_set_state_real", "am_get_state",
    "am_step", "am_step_async", "am_sync", "am_step_profiled", "am_row_passes_async", "am_step_noalloc", "am_launches_per_step", "am_device_bytes", "am_kx_carried",
    "am_status_string",
    "am_last_error", "am_mask_value", "am_ic_bandlimited", "am_spec_read", "am_write_snapshot",
    "am_read_snapshot", "am_append_energy", "am_cli_main", "am_batch_create", "am_batch_destroy",
    "am_batch_set_state", "am_batch_get_state", "am_batch_step", "am_batch_last_error",
    "am_ragged_create", "am_ragged_destroy", "am_ragged_set_state", "am_ragged_get_state", "am_ragged_run",
    "am_ragged_device_bytes", "am_ragged_classes", "am_ragged_set_mode", "am_ragged_last_error",
    "am_server_create", "am_server_submit", "am_server_wait", "am_server_stats", "am_server_destroy",
    "am_footprint_bytes", "am_set_column_shape", "am_column_shape", "am_autotune", "am_set_row_shape",
    "am_row_shape",
]


def status_string(s):
    return lib.am_status_string(s).decode()


def _check(st, h=None, what=""):
    if st != AM_OK:
        detail = lib.am_last_error(h).decode() if h else ""
        raise ActflowError(st, f"{what}: {status_string(st)} {detail}".strip())


def _dptr(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


class Solver:
    """One simulation on the GPU (an am_handle)."""

    def __init__(self, nx, ny, lx, ly, dt, lam, alpha, beta, gamma0=None, gamma2=None,
                 dealias="reference", precision="fp32", if_factors="auto"):
        form = FORM_REFERENCE if gamma0 is None else FORM_GENERAL
        self.precision = _prec(precision)
        self.params = Params(nx, ny, lx, ly, dt, lam, alpha, beta,
                             0.0 if gamma0 is None else gamma0, 0.0 if gamma2 is None else gamma2,
                             form, DEALIAS[dealias] if isinstance(dealias, str) else int(dealias),
                             self.precision, IF_FACTORS[if_factors] if isinstance(if_factors, str)
                             else int(if_factors))
        self.nx, self.ny = nx, ny
        self.h = ctypes.c_void_p()
        _check(lib.am_create(ctypes.byref(self.params), ctypes.byref(self.h)), None, "am_create")
        self.cdtype = np.complex64 if self.precision == FP32 else np.complex128
        self.rdtype = np.float32 if self.precision == FP32 else np.float64

    def close(self):
        if self.h:
            lib.am_destroy(self.h)
            self.h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_stream(self, stream_ptr):
        _check(lib.am_set_stream(self.h, ctypes.c_void_p(stream_ptr)), self.h, "am_set_stream")

    def set_state(self, w_hat, mean=(0.0, 0.0)):
        w = np.ascontiguousarray(w_hat, dtype=self.cdtype)
        assert w.shape == (self.ny, self.nx // 2 + 1)
        m = np.array(mean, dtype=np.float64)
        _check(lib.am_set_state(self.h, w.ctypes.data, _dptr(m)), self.h, "am_set_state")

    def set_state_real(self, w_real, mean=(0.0, 0.0), mask_and_zero_mean=True):
        w = np.ascontiguousarray(w_real, dtype=self.rdtype)
        assert w.shape == (self.ny, self.nx)
        m = np.array(mean, dtype=np.float64)
        _check(lib.am_set_state_real(self.h, w.ctypes.data, _dptr(m), int(mask_and_zero_mean)), self.h,
               "am_set_state_real")

    def get_state(self):
        w = np.zeros((self.ny, self.nx // 2 + 1), dtype=self.cdtype)
        m = np.zeros(2, dtype=np.float64)
        _check(lib.am_get_state(self.h, w.ctypes.data, _dptr(m)), self.h, "am_get_state")
        return w, m

    def step(self, nsteps, energy=True):
        e = np.zeros(max(nsteps, 1), dtype=np.float64)
        nan_at = ctypes.c_int(-1)
        st = lib.am_step(self.h, nsteps, _dptr(e) if energy else None, ctypes.byref(nan_at))
        if st == AM_ERR_NAN:
            raise ActflowError(st, f"NaN after step {nan_at.value}")
        _check(st, self.h, "am_step")
        return e[:nsteps]

    def step_async(self, nsteps):
        _check(lib.am_step_async(self.h, nsteps), self.h, "am_step_async")

    def sync(self):
        _check(lib.am_sync(self.h), self.h, "am_sync")

    def step_profiled(self, nsteps):
        """Per-kernel CUDA-event times (ms) summed over nsteps: (row[4], col[4])."""
        r = np.zeros(4)
        c = np.zeros(4)
        _check(lib.am_step_profiled(self.h, nsteps, _dptr(r), _dptr(c)), self.h, "am_step_profiled")
        return r, c

    def row_passes_async(self, reps=1):
        """Enqueue reps x the step's four row passes alone (for timing; state unchanged)."""
        _check(lib.am_row_passes_async(self.h, reps), self.h, "am_row_passes_async")

    @property
    def launches_per_step(self):
        return lib.am_launches_per_step(self.h)

    @property
    def kx_carried(self):
        """Highest kx the stage fields carry (Nx/4 when the transforms are pruned)."""
        return lib.am_kx_carried(self.h)

    @property
    def device_bytes(self):
        return lib.am_device_bytes(self.h)


class Batch:
    """An ensemble of simulations of one grid advanced together (am_batch)."""

    def __init__(self, params_list):
        n = len(params_list)
        arr = (Params * n)(*params_list)
        self.nx, self.ny, self.n = params_list[0].nx, params_list[0].ny, n
        self.h = ctypes.c_void_p()
        _check(lib.am_batch_create(arr, n, ctypes.byref(self.h)), None, "am_batch_create")

    def _chk(self, st, what):
        if st != AM_OK:
            raise ActflowError(st, f"{what}: {status_string(st)} {lib.am_batch_last_error(self.h).decode()}")

    def close(self):
        if self.h:
            lib.am_batch_destroy(self.h)
            self.h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_state(self, member, w_hat, mean=(0.0, 0.0)):
        w = np.ascontiguousarray(w_hat, dtype=np.complex64)
        m = np.array(mean, dtype=np.float64)
        self._chk(lib.am_batch_set_state(self.h, member, w.ctypes.data, _dptr(m)), "am_batch_set_state")

    def get_state(self, member):
        w = np.zeros((self.ny, self.nx // 2 + 1), dtype=np.complex64)
        m = np.zeros(2)
        self._chk(lib.am_batch_get_state(self.h, member, w.ctypes.data, _dptr(m)), "am_batch_get_state")
        return w, m

    def step(self, nsteps, energy=True):
        e = np.zeros((max(nsteps, 1), self.n))
        nan_m = ctypes.c_int(-1)
        st = lib.am_batch_step(self.h, nsteps, _dptr(e) if energy else None, ctypes.byref(nan_m))
        self._chk(st, "am_batch_step")
        return e[:nsteps]


class Ragged:
    """Simulations of different grids, parameters and step counts advanced together (am_ragged)."""

    def __init__(self, params_list, nsteps):
        n = len(params_list)
        arr = (Params * n)(*params_list)
        steps = (ctypes.c_longlong * n)(*[int(k) for k in nsteps])
        self.shapes = [(p.ny, p.nx // 2 + 1) for p in params_list]
        self.nsteps = [int(k) for k in nsteps]
        self.n = n
        self.h = ctypes.c_void_p()
        _check(lib.am_ragged_create(arr, steps, n, ctypes.byref(self.h)), None, "am_ragged_create")

    def _chk(self, st, what):
        if st != AM_OK:
            raise ActflowError(st, f"{what}: {status_string(st)} {lib.am_ragged_last_error(self.h).decode()}")

    def close(self):
        if self.h:
            lib.am_ragged_destroy(self.h)
            self.h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_state(self, run, w_hat, mean=(0.0, 0.0)):
        w = np.ascontiguousarray(w_hat, dtype=np.complex64)
        assert w.shape == self.shapes[run]
        m = np.array(mean, dtype=np.float64)
        self._chk(lib.am_ragged_set_state(self.h, run, w.ctypes.data, _dptr(m)), "am_ragged_set_state")

    def get_state(self, run):
        w = np.zeros(self.shapes[run], dtype=np.complex64)
        m = np.zeros(2)
        self._chk(lib.am_ragged_get_state(self.h, run, w.ctypes.data, _dptr(m)), "am_ragged_get_state")
        return w, m

    def run(self, energy=True):
        """Advance every run to its step count; returns (energies per run or None, grid-point-steps)."""
        es = [np.zeros(max(k, 1)) for k in self.nsteps] if energy else None
        ptrs = (ctypes.POINTER(ctypes.c_double) * self.n)(*[_dptr(e) for e in es]) if energy else None
        nan_r = ctypes.c_int(-1)
        gps = ctypes.c_longlong(0)
        self._chk(lib.am_ragged_run(self.h, ptrs, ctypes.byref(nan_r), ctypes.byref(gps)), "am_ragged_run")
        return ([e[:k] for e, k in zip(es, self.nsteps)] if energy else None), gps.value

    @property
    def classes(self):
        return lib.am_ragged_classes(self.h)

    def set_mode(self, mode):
        """"worklist" (one launch per pass for every size) or "per_class"."""
        self._chk(lib.am_ragged_set_mode(self.h, {"worklist": 1, "per_class": 0}[mode]), "am_ragged_set_mode")

    @property
    def device_bytes(self):
        return lib.am_ragged_device_bytes(self.h)


class Server:
    """Continuous-batching simulation server on one GPU (am_server)."""

    def __init__(self, hbm_budget_bytes=0, max_active=0, chunk_steps=0, order="arrival", max_active_fp64=0):
        cfg = ServerConfig(int(hbm_budget_bytes), int(max_active), int(chunk_steps), ORDER[order],
                           int(max_active_fp64))
        self.h = ctypes.c_void_p()
        _check(lib.am_server_create(ctypes.byref(cfg), ctypes.byref(self.h)), None, "am_server_create")
        self._jobs = {}

    def submit(self, params, nsteps, seed=0, kmin=1.0, kmax=8.0, rms=0.01, w_hat=None, mean=(0.0, 0.0),
               want_state=True, want_energy=True):
        j = Job()
        j.params = params
        j.nsteps = int(nsteps)
        keep = None
        if w_hat is not None:
            keep = np.ascontiguousarray(w_hat, dtype=np.complex64 if params.precision == FP32 else np.complex128)
            j.w_hat = keep.ctypes.data
        j.mean[0], j.mean[1] = mean
        j.seed, j.kmin, j.kmax, j.rms = int(seed), kmin, kmax, rms
        j.want_state, j.want_energy = int(want_state), int(want_energy)
        jid = ctypes.c_longlong(0)
        _check(lib.am_server_submit(self.h, ctypes.byref(j), ctypes.byref(jid)), None, "am_server_submit")
        self._jobs[jid.value] = (params.nx, params.ny, params.precision, int(nsteps), want_state, want_energy)
        return jid.value

    def wait(self, jid, timeout=-1.0):
        """Result dict of request jid: status, times, mean, state (if kept), energy (if kept)."""
        nx, ny, prec, nsteps, ws, we = self._jobs[jid]
        w = np.zeros((ny, nx // 2 + 1), dtype=np.complex64 if prec == FP32 else np.complex128) if ws else None
        e = np.zeros(max(nsteps, 1)) if we else None
        r = JobResult()
        st = lib.am_server_wait(self.h, jid, timeout, ctypes.byref(r), w.ctypes.data if ws else None,
                                _dptr(e) if we else None)
        if st == AM_ERR_TIMEOUT:
            raise ActflowError(st, f"request {jid}: timed out")
        del self._jobs[jid]
        return {"id": r.id, "status": r.status, "error": r.error.decode(), "t_submit": r.t_submit,
                "t_admit": r.t_admit, "t_done": r.t_done, "mean": np.array(r.mean[:]), "steps_done": r.steps_done,
                "state": w, "energy": e[:nsteps] if we else None}

    def stats(self):
        i = ServerInfo()
        _check(lib.am_server_stats(self.h, ctypes.byref(i)), None, "am_server_stats")
        return {f: getattr(i, f) for f, _ in ServerInfo._fields_}

    def close(self):
        if self.h:
            lib.am_server_destroy(self.h)
            self.h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def footprint_bytes(params):
    return lib.am_footprint_bytes(ctypes.byref(params))


COLUMN_SHAPES = ("wide", "narrow", "wide8")   # "wide8": wide tiles, radix-8 passes (FP32 only)


def set_column_shape(precision, ny, shape):
    """Column-pass launch shape for new simulations of this precision and Ny."""
    prec = _prec(precision)
    _check(lib.am_set_column_shape(prec, ny, COLUMN_SHAPES.index(shape) if isinstance(shape, str) else int(shape)),
           None, "am_set_column_shape")


def column_shape(precision, ny):
    prec = _prec(precision)
    v = lib.am_column_shape(prec, ny)
    return COLUMN_SHAPES[v] if v >= 0 else None


# row-pass shapes: the three inverse transforms in lockstep (radix 8), or one
# after another with shared-memory stashes ("sequence": FP32 radix 16,
# double-float radix 8; Nx >= 1024), or lockstep with the input rows fetched
# by tensor-map copies ("lockstep-tma": FP32, Nx >= 128)
ROW_SHAPES = ("lockstep", "sequence", "lockstep-tma")


def set_row_shape(precision, nx, shape):
    """Row-pass launch shape for new simulations of this precision and Nx."""
    prec = _prec(precision)
    _check(lib.am_set_row_shape(prec, nx, ROW_SHAPES.index(shape) if isinstance(shape, str) else int(shape)),
           None, "am_set_row_shape")


def row_shape(precision, nx):
    prec = _prec(precision)
    v = lib.am_row_shape(prec, nx)
    return ROW_SHAPES[v] if v >= 0 else None


def autotune(params, nsteps=20):
    """Time every column-pass shape built for `params`' precision on this GPU
    and keep the fastest, then every row-pass shape with it.  Returns
    ({column shape: ms per step}, chosen column shape, {row shape: ms}, chosen row shape)."""
    mc = np.zeros(len(COLUMN_SHAPES))
    mr = np.zeros(len(ROW_SHAPES))
    _check(lib.am_autotune(ctypes.byref(params), int(nsteps), _dptr(mc), _dptr(mr)), None, "am_autotune")
    tc = {name: float(t) for name, t in zip(COLUMN_SHAPES, mc) if t >= 0}
    tr = {name: float(t) for name, t in zip(ROW_SHAPES, mr) if t >= 0}
    return tc, column_shape(params.precision, params.ny), tr, row_shape(params.precision, params.nx)


def make_params(nx, ny, lx, ly, dt, lam, alpha, beta, gamma0=None, gamma2=None, dealias="reference",
                precision="fp32", if_factors="auto"):
    form = FORM_REFERENCE if gamma0 is None else FORM_GENERAL
    return Params(nx, ny, lx, ly, dt, lam, alpha, beta, 0.0 if gamma0 is None else gamma0,
                  0.0 if gamma2 is None else gamma2, form,
                  DEALIAS[dealias] if isinstance(dealias, str) else int(dealias),
                  _prec(precision),
                  IF_FACTORS[if_factors] if isinstance(if_factors, str) else int(if_factors))


def mask_value(nx, ny, dealias, ix, iy):
    return lib.am_mask_value(nx, ny, DEALIAS[dealias] if isinstance(dealias, str) else int(dealias), ix, iy)


def ic_bandlimited(nx, ny, seed, kmin=1.0, kmax=8.0, rms=0.01):
    w = np.zeros((ny, nx // 2 + 1), dtype=np.complex128)
    _check(lib.am_ic_bandlimited(nx, ny, seed, kmin, kmax, rms, w.ctypes.data_as(ctypes.POINTER(ctypes.c_double))),
           None, "am_ic_bandlimited")
    return w


def read_spec(directory):
    s = Spec()
    err = ctypes.create_string_buffer(1024)
    st = lib.am_spec_read(directory.encode(), ctypes.byref(s), err, 1024)
    if st != AM_OK:
        raise ActflowError(st, err.value.decode())
    return s


def write_snapshot(path, w_hat, mean, precision="fp32"):
    prec = _prec(precision)
    w = np.ascontiguousarray(w_hat, dtype=np.complex64 if prec == FP32 else np.complex128)
    ny, nxh = w.shape
    m = np.array(mean, dtype=np.float64)
    _check(lib.am_write_snapshot(path.encode(), 2 * (nxh - 1), ny, prec, w.ctypes.data, _dptr(m)), None,
           "am_write_snapshot")


def read_snapshot(path, nx, ny, precision="fp32"):
    prec = _prec(precision)
    w = np.zeros((ny, nx // 2 + 1), dtype=np.complex64 if prec == FP32 else np.complex128)
    m = np.zeros(2, dtype=np.float64)
    _check(lib.am_read_snapshot(path.encode(), nx, ny, prec, w.ctypes.data, _dptr(m)), None, "am_read_snapshot")
    return w, m


def append_energy(path, m0, dt, energy, precision="fp32"):
    prec = _prec(precision)
    e = np.ascontiguousarray(energy, dtype=np.float64)
    _check(lib.am_append_energy(path.encode(), m0, len(e), dt, _dptr(e), prec), None, "am_append_energy")


def cli_main(args):
    """Run the drop-in program in-process: cli_main(["actflow", dir])."""
    argv = (ctypes.c_char_p * len(args))(*[a.encode() for a in args])
    return lib.am_cli_main(len(args), argv)
