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
        src = os.path.join(HERE, "amca_oracle.c")
        if not os.path.exists(LIB) or (os.path.exists(src) and os.path.getmtime(src) > os.path.getmtime(LIB)):
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
        _lib.amca_oracle_run_remelt.argtypes = [ctypes.POINTER(RemeltParams), ctypes.c_int, ctypes.c_char_p, vp, vp,
                                                vp, vp, vp, vp, ctypes.POINTER(RemeltResult), ctypes.c_char_p,
                                                ctypes.c_int]
        _lib.amca_oracle_run_remelt.restype = ctypes.c_int
        _lib.amca_oracle_is_in_element.argtypes = [vp, vp, ctypes.c_double, ctypes.c_int, vp]
        _lib.amca_oracle_is_in_element.restype = ctypes.c_int
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


# ---------------------------------------------------------------------------
# FE-coupled remelting realm
# ---------------------------------------------------------------------------
class RemeltParams(ctypes.Structure):
    _fields_ = [("nx", ctypes.c_int), ("ny", ctypes.c_int), ("nz", ctypes.c_int), ("x0", ctypes.c_double),
                ("y0", ctypes.c_double), ("z0", ctypes.c_double), ("h", ctypes.c_double), ("Tm", ctypes.c_double),
                ("Ts", ctypes.c_double), ("Tnuc_min", ctypes.c_double), ("a1", ctypes.c_double),
                ("a2", ctypes.c_double), ("a3", ctypes.c_double), ("b1", ctypes.c_double), ("b2", ctypes.c_double),
                ("b3", ctypes.c_double), ("time_step_factor_ca", ctypes.c_double), ("trunc_coeff", ctypes.c_double),
                ("cutoff_factor", ctypes.c_double), ("initial_melted", ctypes.c_int), ("nucleation", ctypes.c_int),
                ("ns", ctypes.c_double), ("mu_s", ctypes.c_double), ("sigma_s", ctypes.c_double),
                ("nv", ctypes.c_double), ("mu_v", ctypes.c_double), ("sigma_v", ctypes.c_double),
                ("seed", ctypes.c_uint), ("shuffle_vtr", ctypes.c_int), ("microstructure", ctypes.c_char_p),
                ("load_seeds", ctypes.c_int), ("bin", ctypes.c_int * 3), ("tolerance", ctypes.c_double),
                ("max_iter", ctypes.c_int), ("void_temperature", ctypes.c_double), ("frames", ctypes.c_char_p),
                ("title_lines", ctypes.c_int), ("subtitle_lines", ctypes.c_int), ("length_scale", ctypes.c_double),
                ("time_scale", ctypes.c_double), ("offset", ctypes.c_double * 3), ("final_time", ctypes.c_double)]


class RemeltResult(ctypes.Structure):
    _fields_ = [("steps", ctypes.c_int), ("time", ctypes.c_double), ("last_dt", ctypes.c_double),
                ("num_grains", ctypes.c_int64), ("num_orient", ctypes.c_int64), ("num_sites", ctypes.c_int64),
                ("tests", ctypes.c_int64), ("nodes", ctypes.c_int64), ("elements", ctypes.c_int64),
                ("frames_read", ctypes.c_int64), ("frames_exhausted", ctypes.c_int), ("loop_seconds", ctypes.c_double)]

    def as_dict(self) -> dict:
        return {k: getattr(self, k) for k, _ in self._fields_}


def remelt_params_of(case, workdir: str) -> RemeltParams:
    """Oracle parameters of an amca3d_gb300.decks.RemeltCase whose files
    (frames, restart file) lie in workdir, as the reference reads them."""
    import numpy as _np

    nx, ny, nz = case.cells
    p = RemeltParams()
    p.nx, p.ny, p.nz = nx, ny, nz
    p.x0, p.y0, p.z0 = case.origin
    p.h = case.cell_size
    p.Tm, p.Ts = case.melting_temperature, case.solidus_temperature
    p.Tnuc_min = case.solidus_temperature if case.min_nucleation_temperature is None else case.min_nucleation_temperature
    p.a1, p.a2, p.a3 = case.a
    p.b1, p.b2, p.b3 = 1.0, 2.0, 3.0
    p.time_step_factor_ca = 0.2 if case.time_step_factor_ca is None else case.time_step_factor_ca
    p.trunc_coeff = float(_np.float32(_np.sqrt(_np.float32(3.0))))
    p.cutoff_factor = 1.0e8 if case.cutoff_factor is None else case.cutoff_factor
    p.initial_melted = 1 if case.has_been_melted else 0
    p.nucleation = 1 if case.nucleation else 0
    p.ns, p.mu_s, p.sigma_s = case.surface
    p.nv, p.mu_v, p.sigma_v = case.bulk
    p.seed = case.seed
    p.shuffle_vtr = 1 if case.shuffle_vtr else 0
    p.microstructure = None if case.microstructure == "random" else os.path.join(workdir, case.microstructure).encode()
    p.load_seeds = 1 if case.load_seeds else 0
    p.bin[0], p.bin[1], p.bin[2] = case.bin_size
    p.tolerance = case.tolerance
    p.max_iter = case.max_iterations
    p.void_temperature = -1.0e8 if case.void_temperature is None else case.void_temperature
    p.frames = os.path.join(workdir, case.frames_file).encode()
    p.title_lines, p.subtitle_lines = case.lines_for_title, case.lines_for_subtitle
    p.length_scale, p.time_scale = case.length_scale, case.time_scale
    p.offset[0], p.offset[1], p.offset[2] = case.offset
    p.final_time = case.termination_time
    return p


def run_remelt(case, workdir: str, max_steps: int = -1, dump: Optional[str] = None, fields: bool = True) -> dict:
    """Run the remelting oracle on a RemeltCase prepared in workdir."""
    p = remelt_params_of(case, workdir)
    n = case.n_ghost
    arr = dict(orient=np.empty(n, np.int32), grain=np.empty(n, np.int32), T=np.empty(n, np.float64),
               melted=np.empty(n, np.uint8), cooling=np.empty(n, np.uint8), flag=np.empty(n, np.uint8)) if fields else {}
    r = RemeltResult()
    err = ctypes.create_string_buffer(512)
    rc = lib().amca_oracle_run_remelt(ctypes.byref(p), int(max_steps), dump.encode() if dump else None,
                                      *(_p(arr.get(k)) for k in ("orient", "grain", "T", "melted", "cooling", "flag")),
                                      ctypes.byref(r), err, 512)
    if rc != 0:
        raise RuntimeError(f"remelting oracle failed ({rc}): {err.value.decode()}")
    out = r.as_dict()
    out.update(arr)
    return out


def is_in_element(node_xyz, point, tolerance: float = 1e-16, max_iter: int = 20):
    nx = np.ascontiguousarray(node_xyz, np.float64).reshape(24)
    pt = np.ascontiguousarray(point, np.float64).reshape(3)
    para = np.empty(3, np.float64)
    ok = lib().amca_oracle_is_in_element(_p(nx), _p(pt), float(tolerance), int(max_iter), _p(para))
    return bool(ok), para
