"""ctypes wrapper of the float64 C port (test infrastructure only)."""

import ctypes
import os
import time

import numpy as np

from . import build_port

_LIB = None
FIELDS = {"lotka_volterra": 0, "van_der_pol": 1, "fitzhugh_nagumo": 2}
SOLVERS = {"none": 0, "mle": 1, "dynamic": 2}
CONTROLS = {"integral": 0, "proportional_integral": 1}


def load():
    global _LIB
    if _LIB is None:
        build_port.build()
        lib = ctypes.CDLL(build_port.LIB)
        P = ctypes.POINTER
        lib.pdq_port_solve_iso.restype = ctypes.c_int
        lib.pdq_port_solve_iso.argtypes = [
            ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_double, ctypes.c_double,
            ctypes.c_double, ctypes.c_double, ctypes.c_double, ctypes.c_int64,
            P(ctypes.c_double), P(ctypes.c_double), ctypes.c_int,
            P(ctypes.c_double), P(ctypes.c_double), P(ctypes.c_double), P(ctypes.c_int), P(ctypes.c_int),
        ]
        _LIB = lib
    return _LIB


def solve_iso_terminal(field, params, y0, nu, solver="mle", control="integral", atol=1e-6, rtol=1e-6, t0=0.0, t1=50.0, dt0=0.1, threads=None):
    """Terminal values of B instances; returns dict of numpy arrays."""
    lib = load()
    params = np.ascontiguousarray(np.asarray(params, dtype=np.float64))
    y0 = np.ascontiguousarray(np.asarray(y0, dtype=np.float64))
    B = y0.shape[0]
    n = nu + 1
    out = {
        "mean": np.zeros((B, n, 2)),
        "chol": np.zeros((B, n, n)),
        "output_scale": np.zeros(B),
        "num_steps": np.zeros(B, dtype=np.int32),
        "num_attempts": np.zeros(B, dtype=np.int32),
    }
    dp = ctypes.POINTER(ctypes.c_double)
    ip = ctypes.POINTER(ctypes.c_int)
    st = lib.pdq_port_solve_iso(
        FIELDS[field], nu, SOLVERS[solver], CONTROLS[control], atol, rtol, t0, t1, dt0, B,
        params.ctypes.data_as(dp), y0.ctypes.data_as(dp), int(threads or os.cpu_count() or 1),
        out["mean"].ctypes.data_as(dp), out["chol"].ctypes.data_as(dp), out["output_scale"].ctypes.data_as(dp),
        out["num_steps"].ctypes.data_as(ip), out["num_attempts"].ctypes.data_as(ip),
    )
    if st != 0:
        raise RuntimeError("port failed")
    return out


def time_lv_ensemble(params, y0, threads=None):
    """Wall time (s) of terminal-value MLE solves of the LV ensemble workload."""
    t = time.perf_counter()
    solve_iso_terminal("lotka_volterra", params, y0, 4, solver="mle", threads=threads)
    return time.perf_counter() - t
