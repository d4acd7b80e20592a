"""ctypes front end of the oracle (CPU restatement of the reference step).

TEST INFRASTRUCTURE ONLY.  Only ``tests/``, ``__graft_entry__.smoke()`` and the
CPU-baseline leg of ``bench.py`` may import this package, and only as the
checker.  The product (the CUDA solver behind ``include/actflow.h``) never
imports, links or calls it.

The library is built from ``actflow_oracle.c`` / ``oracle_core.h`` by
``oracle/Makefile`` (``build()`` in ``__graft_entry__`` runs it).
"""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "lib", "liborc.so")


class OrcParams(ctypes.Structure):
    _fields_ = [
        ("nx", ctypes.c_int), ("ny", ctypes.c_int),
        ("lx", ctypes.c_double), ("ly", ctypes.c_double), ("dt", ctypes.c_double),
        ("lam", ctypes.c_double), ("alpha", ctypes.c_double), ("beta", ctypes.c_double),
        ("gamma0", ctypes.c_double), ("gamma2", ctypes.c_double),
        ("form", ctypes.c_int), ("dealias", ctypes.c_int), ("if_double", ctypes.c_int),
    ]


DEALIAS = {"reference": 0, "half": 1, "none": 2}

_lib = None


def build():
    subprocess.run(["make", "-s", "-C", HERE], check=True)


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        L = ctypes.CDLL(LIB_PATH)
        dp = ctypes.POINTER(ctypes.c_double)
        fp = ctypes.POINTER(ctypes.c_float)
        L.orc_run_f32.argtypes = [ctypes.POINTER(OrcParams), fp, fp, ctypes.c_int, dp, ctypes.c_int]
        L.orc_run_f64.argtypes = [ctypes.POINTER(OrcParams), dp, dp, ctypes.c_int, dp, ctypes.c_int]
        L.orc_rfft2_f32.argtypes = [ctypes.c_int, ctypes.c_int, fp, fp]
        L.orc_rfft2_f64.argtypes = [ctypes.c_int, ctypes.c_int, dp, dp]
        L.orc_irfft2_f32.argtypes = [ctypes.c_int, ctypes.c_int, fp, fp]
        L.orc_irfft2_f64.argtypes = [ctypes.c_int, ctypes.c_int, dp, dp]
        L.orc_mask.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, fp]
        L.orc_mask_value.argtypes = [ctypes.c_int] * 5
        L.orc_num_threads.restype = ctypes.c_int
        _lib = L
    return _lib


def make_params(nx, ny, lx, ly, dt, lam, alpha, beta, gamma0=None, gamma2=None, dealias="reference",
                if_double=False):
    """if_double: integrating factors evaluated in double and rounded once to
    the run's precision (the solver's precision form) instead of in that
    precision as lin_func does."""
    form = 0 if gamma0 is None else 1
    return OrcParams(nx, ny, lx, ly, dt, lam, alpha, beta,
                     0.0 if gamma0 is None else gamma0, 0.0 if gamma2 is None else gamma2,
                     form, DEALIAS[dealias] if isinstance(dealias, str) else int(dealias), 1 if if_double else 0)


def run(params, w_hat, mean, nsteps, precision="f64", nthreads=0):
    """Advance (w_hat [ny][nx/2+1] complex, mean[2]) by nsteps steps.

    Returns (w_hat, mean, energy[nsteps]); energy[m] is the energy of the state
    at the start of step m, as the reference's energy.txt records it.
    """
    if precision == "f32":
        w = np.ascontiguousarray(w_hat, dtype=np.complex64).copy()
        m = np.array(mean, dtype=np.float32)
        e = np.zeros(max(nsteps, 1), dtype=np.float64)
        rc = lib().orc_run_f32(ctypes.byref(params), w.ctypes.data_as(ctypes.POINTER(ctypes.c_float)),
                               m.ctypes.data_as(ctypes.POINTER(ctypes.c_float)), nsteps,
                               e.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), nthreads)
    else:
        w = np.ascontiguousarray(w_hat, dtype=np.complex128).copy()
        m = np.array(mean, dtype=np.float64)
        e = np.zeros(max(nsteps, 1), dtype=np.float64)
        rc = lib().orc_run_f64(ctypes.byref(params), w.ctypes.data_as(ctypes.POINTER(ctypes.c_double)),
                               m.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), nsteps,
                               e.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), nthreads)
    if rc != 0:
        raise ValueError("oracle: unsupported grid (power-of-two sizes only)")
    return w, m, e[:nsteps]


def rfft2(x, precision="f64"):
    ny, nx = x.shape
    if precision == "f32":
        a = np.ascontiguousarray(x, dtype=np.float32)
        out = np.zeros((ny, nx // 2 + 1), dtype=np.complex64)
        lib().orc_rfft2_f32(nx, ny, a.ctypes.data_as(ctypes.POINTER(ctypes.c_float)),
                            out.ctypes.data_as(ctypes.POINTER(ctypes.c_float)))
    else:
        a = np.ascontiguousarray(x, dtype=np.float64)
        out = np.zeros((ny, nx // 2 + 1), dtype=np.complex128)
        lib().orc_rfft2_f64(nx, ny, a.ctypes.data_as(ctypes.POINTER(ctypes.c_double)),
                            out.ctypes.data_as(ctypes.POINTER(ctypes.c_double)))
    return out


def irfft2(X, nx, precision="f64"):
    ny = X.shape[0]
    if precision == "f32":
        a = np.ascontiguousarray(X, dtype=np.complex64)
        out = np.zeros((ny, nx), dtype=np.float32)
        lib().orc_irfft2_f32(nx, ny, a.ctypes.data_as(ctypes.POINTER(ctypes.c_float)),
                             out.ctypes.data_as(ctypes.POINTER(ctypes.c_float)))
    else:
        a = np.ascontiguousarray(X, dtype=np.complex128)
        out = np.zeros((ny, nx), dtype=np.float64)
        lib().orc_irfft2_f64(nx, ny, a.ctypes.data_as(ctypes.POINTER(ctypes.c_double)),
                             out.ctypes.data_as(ctypes.POINTER(ctypes.c_double)))
    return out


def mask(nx, ny, mode):
    out = np.zeros((ny, nx // 2 + 1), dtype=np.float32)
    lib().orc_mask(nx, ny, DEALIAS[mode] if isinstance(mode, str) else int(mode),
                   out.ctypes.data_as(ctypes.POINTER(ctypes.c_float)))
    return out


def num_threads():
    return lib().orc_num_threads()
