"""ctypes binding of the C oracle (oracle/amca_oracle.c).

TEST INFRASTRUCTURE ONLY: used by tests/, __graft_entry__.smoke() and the
CPU-baseline leg of bench.py as the checker. The product never imports it.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
from typing import Optional

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "_build", "libamca_oracle.so")


class PlainParams(ctypes.Structure):
    _fields_ = [("nx", ctypes.c_int), ("ny", ctypes.c_int), ("nz", ctypes.c_int), ("x0", ctypes.c_double),
                ("y0", ctypes.c_double), ("z0", ctypes.c_double), ("h", ctypes.c_double), ("ns", ctypes.c_double),
                ("mu_s", ctypes.c_double), ("sigma_s", ctypes.c_double), ("nv", ctypes.c_double),
                ("mu_v", ctypes.c_double), ("sigma_v", ctypes.c_double), ("seed", ctypes.c_uint),
                ("T0", ctypes.c_double), ("Tm", ctypes.c_double), ("Tdot", ctypes.c_double), ("a1", ctypes.c_double),
                ("a2", ctypes.c_double), ("a3", ctypes.c_double), ("max_dt", ctypes.c_double),
                ("final_time", ctypes.c_double), ("time_step_factor", ctypes.c_double),
                ("trunc_coeff", ctypes.c_double), ("shuffle_vtr", ctypes.c_int)]


class Result(ctypes.Structure):
    _fields_ = [("steps", ctypes.c_int), ("time", ctypes.c_double), ("last_dt", ctypes.c_double),
                ("num_grains", ctypes.c_int64), ("num_orient", ctypes.c_int64), ("liquid_cells", ctypes.c_int64),
                ("active_grains", ctypes.c_int64), ("tests", ctypes.c_int64), ("num_sites", ctypes.c_int64)]

    def as_dict(self) -> dict:
        return {k: getattr(self, k) for k, _ in self._fields_}


_lib = None


def build() -> str:
    subprocess.run(["make", "-s", "-C", HERE, "port"], check=True)
    return LIB


def lib() -> ctypes.CDLL:
    global _lib
    if _lib is None:
        if not os.path.exists(LIB):
            build()
        _lib = ctypes.CDLL(LIB)
        vp = ctypes.c_void_p
        _lib.amca_oracle_run_plain.argtypes = [ctypes.POINTER(PlainParams), ctypes.c_int, vp, vp, vp, vp,
                                               ctypes.c_int64, ctypes.POINTER(Result)]
        _lib.amca_oracle_run_plain.restype = ctypes.c_int
        _lib.amca_oracle_normal_draws.argtypes = [ctypes.c_double, ctypes.c_double, ctypes.c_int, vp]
        _lib.amca_oracle_orientation.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, vp, vp]
        _lib.amca_oracle_rotation.argtypes = [vp, vp]
        _lib.amca_oracle_is_captured.argtypes = [vp, vp, ctypes.c_double]
        _lib.amca_oracle_is_captured.restype = ctypes.c_int
        _lib.amca_oracle_capture.argtypes = [vp, vp, ctypes.c_double, ctypes.c_double, ctypes.c_double, vp]
    return _lib


def params_of(case) -> PlainParams:
    """Oracle parameters of an amca3d_gb300.decks.PlainCase."""
    nx, ny, nz = case.cells
    return PlainParams(nx, ny, nz, case.origin[0], case.origin[1], case.origin[2], case.cell_size,
                       case.surface[0], case.surface[1], case.surface[2], case.bulk[0], case.bulk[1], case.bulk[2],
                       case.seed, case.initial_temperature, case.melting_temperature, case.t_dot, case.a[0], case.a[1],
                       case.a[2], case.time_step, case.termination_time,
                       0.2 if case.time_step_factor_ca is None else case.time_step_factor_ca, case.trunc_coeff(),
                       1 if case.shuffle_vtr else 0)


def _p(a: Optional[np.ndarray]):
    return None if a is None else a.ctypes.data_as(ctypes.c_void_p)


def run_plain(case, max_steps: int = -1, fields: bool = True, euler_cap: int = 0) -> dict:
    """Run the oracle on a PlainCase. Returns the result counters and, with
    fields=True, the ghost-inclusive orientation / grain / site-dTc fields."""
    p = params_of(case)
    n = case.n_ghost
    o = np.empty(n, np.int32) if fields else None
    g = np.empty(n, np.int32) if fields else None
    d = np.empty(n, np.float64) if fields else None
    e = np.empty((max(euler_cap, 0), 3), np.float64) if euler_cap > 0 else None
    r = Result()
    rc = lib().amca_oracle_run_plain(ctypes.byref(p), int(max_steps), _p(o), _p(g), _p(d), _p(e),
                                     ctypes.c_int64(euler_cap), ctypes.byref(r))
    if rc != 0:
        raise RuntimeError(f"oracle failed with {rc}")
    out = r.as_dict()
    if fields:
        out.update(orient=o, grain=g, site_dtc=d)
    if e is not None:
        out["euler"] = e[: min(euler_cap, r.num_orient)]
    return out


def normal_draws(mean: float, sigma: float, n: int) -> np.ndarray:
    out = np.empty(n, np.float64)
    lib().amca_oracle_normal_draws(mean, sigma, n, _p(out))
    return out


def rotation(euler) -> np.ndarray:
    e = np.ascontiguousarray(euler, np.float64)
    m = np.empty(9, np.float64)
    lib().amca_oracle_rotation(_p(e), _p(m))
    return m


def is_captured(l2g, gc, length: float) -> bool:
    m = np.ascontiguousarray(l2g, np.float64)
    g = np.ascontiguousarray(gc, np.float64)
    return bool(lib().amca_oracle_is_captured(_p(m), _p(g), float(length)))


def capture(l2g, gc, length: float, h: float, trunc: float) -> np.ndarray:
    m = np.ascontiguousarray(l2g, np.float64)
    g = np.ascontiguousarray(gc, np.float64)
    out = np.empty(4, np.float64)
    lib().amca_oracle_capture(_p(m), _p(g), float(length), float(h), float(trunc), _p(out))
    return out
