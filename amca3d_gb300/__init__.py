"""GB300 CA timestep of AMCA3D behind the reference's own input surface.

Python binding (ctypes) of the C ABI in ``include/amca3d.h``. The compute
path is the in-tree ``libamca3d.so`` (hand-written sm_103a CUDA); there is no
CPU fallback — importing works anywhere, but every call that needs the GPU
fails loudly if the library or the device is missing.

    realm = CellularAutomataRealm(deck_text, seed=0)
    realm.initialize()
    realm.run()                       # until solid / termination_time
    grain_id = realm.field("orientation_id")

The method names follow the reference's ``CellularAutomataManager`` interface
(CA/include/CellularAutomataManager.h:20-246): ``initialize``,
``single_integration_step`` (one ``calculate_time_step`` +
``single_integration_step``), ``time_integration``.
"""
from __future__ import annotations

import ctypes
import os
from typing import Optional

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libamca3d.so")

AMCA_OK = 0
FIELD_IDS = {"orientation_id": 0, "grain_id": 1, "site_undercooling": 2, "temperature": 3, "melted": 4,
             "cooling": 5, "liquid_neighbour": 6}
FIELD_DTYPES = {"orientation_id": np.int32, "grain_id": np.int32, "site_undercooling": np.float64,
                "temperature": np.float64, "melted": np.uint8, "cooling": np.uint8, "liquid_neighbour": np.uint8}
_ERRORS = {-1: "bad argument", -2: "deck parse error", -3: "CUDA error", -4: "call out of order",
           -5: "device-side error", -6: "output error"}


class AmcaError(RuntimeError):
    def __init__(self, code: int, message: str):
        super().__init__(f"{_ERRORS.get(code, code)}: {message}")
        self.code = code


class _Opts(ctypes.Structure):
    _fields_ = [("device", ctypes.c_int), ("seed", ctypes.c_uint), ("write_outputs", ctypes.c_int),
                ("workdir", ctypes.c_char_p)]


class Stats(ctypes.Structure):
    _fields_ = [("step", ctypes.c_int64), ("time", ctypes.c_double), ("dt", ctypes.c_double),
                ("liquid_cells", ctypes.c_int64), ("grains", ctypes.c_int64), ("orientations", ctypes.c_int64),
                ("active", ctypes.c_int64), ("sites", ctypes.c_int64), ("cells", ctypes.c_int64),
                ("tests", ctypes.c_int64), ("tests_fp64", ctypes.c_int64), ("generations", ctypes.c_int64),
                ("done", ctypes.c_int32), ("reserved", ctypes.c_int32), ("kernel_ms", ctypes.c_double),
                ("launches", ctypes.c_int64), ("sites_scanned", ctypes.c_int64), ("nucleations", ctypes.c_int64),
                ("captures", ctypes.c_int64), ("active_grown", ctypes.c_int64),
                ("grains_processed", ctypes.c_int64), ("algorithmic_bytes", ctypes.c_double),
                ("h2d_bytes", ctypes.c_int64), ("d2h_bytes", ctypes.c_int64), ("phase_ms", ctypes.c_double * 9),
                ("detail_ms", ctypes.c_double * 16), ("keys_scanned", ctypes.c_int64),
                ("decrements", ctypes.c_int64), ("zero_events", ctypes.c_int64), ("compactions", ctypes.c_int64),
                ("reference_walked", ctypes.c_int64), ("step_bytes", ctypes.c_double)]

    def as_dict(self) -> dict:
        d = {k: getattr(self, k) for k, _ in self._fields_}
        d["phase_ms"] = list(d["phase_ms"])
        d["detail_ms"] = list(d["detail_ms"])
        return d


# every entry point declared in include/amca3d.h
EXPORTS = ("amca_create", "amca_get_grid", "amca_prepare", "amca_get_sites", "amca_initialize", "amca_step",
           "amca_run", "amca_get_field", "amca_get_orientations", "amca_write_outputs", "amca_get_stats",
           "amca_final_grain_count", "amca_reset", "amca_host_alloc", "amca_host_free", "amca_envelope_eval",
           "amca_plain_run_noalloc", "amca_selftest_barrier", "amca_release_cached_memory", "amca_set_fe_frames", "amca_set_rosenthal_frames", "amca_set_microstructure",
           "amca_step_coupled", "amca_run_until", "amca_set_nodal_temperatures",
           "amca_set_scan_frames", "amca_set_thermal_frames", "amca_get_frame_stats", "amca_thermal_create",
           "amca_thermal_train", "amca_thermal_eval", "amca_thermal_gradients", "amca_thermal_param_count",
           "amca_thermal_get_params", "amca_thermal_set_params", "amca_thermal_get_encoding", "amca_thermal_frames",
           "amca_thermal_last_error", "amca_thermal_destroy",
           "amca_batch_create", "amca_batch_run", "amca_batch_tune", "amca_batch_set_layout", "amca_batch_get_layout",
           "amca_batch_get_stats",
           "amca_batch_last_error",
           "amca_batch_destroy", "amca_last_error", "amca_destroy")


class Rosenthal(ctypes.Structure):
    """amca_rosenthal of include/amca3d.h: synthetic frames generated on the GPU."""
    _fields_ = [("origin", ctypes.c_double * 3), ("spacing", ctypes.c_double), ("nodes", ctypes.c_int32 * 3),
                ("frames", ctypes.c_int32), ("length_scale", ctypes.c_double), ("frame_dt", ctypes.c_double),
                ("time_scale", ctypes.c_double), ("time_offset", ctypes.c_double), ("power", ctypes.c_double),
                ("absorptivity", ctypes.c_double), ("speed", ctypes.c_double), ("conductivity", ctypes.c_double),
                ("diffusivity", ctypes.c_double), ("t0", ctypes.c_double), ("t_cap", ctypes.c_double),
                ("x_start", ctypes.c_double), ("y_line", ctypes.c_double), ("z_top", ctypes.c_double),
                ("void_above_set", ctypes.c_int32), ("void_above", ctypes.c_double), ("t_void", ctypes.c_double)]


class Scan(ctypes.Structure):
    """amca_scan of include/amca3d.h: frames of a raster scan (FE field or model)."""
    _fields_ = [("origin", ctypes.c_double * 3), ("spacing", ctypes.c_double), ("nodes", ctypes.c_int32 * 3),
                ("frames", ctypes.c_int32), ("length_scale", ctypes.c_double), ("frame_dt", ctypes.c_double),
                ("time_scale", ctypes.c_double), ("time_offset", ctypes.c_double), ("power", ctypes.c_double),
                ("absorptivity", ctypes.c_double), ("speed", ctypes.c_double), ("conductivity", ctypes.c_double),
                ("diffusivity", ctypes.c_double), ("t0", ctypes.c_double), ("t_cap", ctypes.c_double),
                ("x_start", ctypes.c_double), ("x_turn", ctypes.c_double), ("y_line", ctypes.c_double),
                ("z_top", ctypes.c_double), ("hatch", ctypes.c_double), ("track_time", ctypes.c_double),
                ("ntracks", ctypes.c_int32)]

    @classmethod
    def of(cls, **kw) -> "Scan":
        s = cls()
        for k, v in kw.items():
            if k in ("origin", "nodes"):
                for a in range(3):
                    getattr(s, k)[a] = v[a]
            else:
                setattr(s, k, v)
        return s


class ThermalSpec(ctypes.Structure):
    """amca_thermal_spec of include/amca3d.h."""
    _fields_ = [("power_lo", ctypes.c_double), ("power_hi", ctypes.c_double), ("speed_lo", ctypes.c_double),
                ("speed_hi", ctypes.c_double), ("absorptivity", ctypes.c_double), ("conductivity", ctypes.c_double),
                ("diffusivity", ctypes.c_double), ("t0", ctypes.c_double), ("t_cap", ctypes.c_double),
                ("window_lo", ctypes.c_double * 3), ("window_hi", ctypes.c_double * 3),
                ("near_lo", ctypes.c_double * 3), ("near_hi", ctypes.c_double * 3), ("near_fraction", ctypes.c_double),
                ("shell_lo", ctypes.c_double), ("shell_hi", ctypes.c_double), ("shell_fraction", ctypes.c_double),
                ("fourier_sigma", ctypes.c_double), ("fourier_sigma_pv", ctypes.c_double),
                ("log_output", ctypes.c_int32), ("t_shift", ctypes.c_double), ("t_scale", ctypes.c_double),
                ("seed", ctypes.c_uint64)]


class ThermalTrainStats(ctypes.Structure):
    _fields_ = [("steps", ctypes.c_int64), ("samples_seen", ctypes.c_int64), ("first_loss", ctypes.c_double),
                ("last_loss", ctypes.c_double), ("ms", ctypes.c_double)]


class BatchStats(ctypes.Structure):
    """amca_batch_stats of include/amca3d.h."""
    _fields_ = [("realms", ctypes.c_int32), ("team_size", ctypes.c_int32), ("teams", ctypes.c_int32),
                ("max_blocks", ctypes.c_int32), ("graph", ctypes.c_int32), ("n_tuned", ctypes.c_int32),
                ("runs", ctypes.c_int64), ("last_ms", ctypes.c_double), ("total_ms", ctypes.c_double),
                ("cell_updates", ctypes.c_int64), ("tuned_team", ctypes.c_int32 * 8),
                ("tuned_ms", ctypes.c_double * 8), ("mixed_ms", ctypes.c_double), ("grid_blocks", ctypes.c_int32),
                ("n_classes", ctypes.c_int32), ("class_team", ctypes.c_int32 * 8),
                ("class_teams", ctypes.c_int32 * 8), ("class_realms", ctypes.c_int32 * 8)]

    def as_dict(self) -> dict:
        d = {k: getattr(self, k) for k, _ in self._fields_ if not k.startswith(("tuned_", "class_"))}
        d["tuned"] = {int(self.tuned_team[i]): float(self.tuned_ms[i]) for i in range(self.n_tuned)}
        d["classes"] = [{"team_size": int(self.class_team[i]), "teams": int(self.class_teams[i]),
                         "realms": int(self.class_realms[i])} for i in range(self.n_classes)]
        return d


class PlainParams(ctypes.Structure):
    """amca_plain_params of include/amca3d.h."""
    _fields_ = [("nx", ctypes.c_int32), ("ny", ctypes.c_int32), ("nz", ctypes.c_int32), ("x0", ctypes.c_double),
                ("y0", ctypes.c_double), ("z0", ctypes.c_double), ("h", ctypes.c_double), ("T0", ctypes.c_double),
                ("Tm", ctypes.c_double), ("Tdot", ctypes.c_double), ("a1", ctypes.c_double), ("a2", ctypes.c_double),
                ("a3", ctypes.c_double), ("max_dt", ctypes.c_double), ("final_time", ctypes.c_double),
                ("time_step_factor", ctypes.c_double), ("trunc_coeff", ctypes.c_double)]


class PlainResult(ctypes.Structure):
    _fields_ = [("steps", ctypes.c_int64), ("time", ctypes.c_double), ("grains", ctypes.c_int64),
                ("orientations", ctypes.c_int64), ("liquid_cells", ctypes.c_int64), ("done", ctypes.c_int32)]

_lib = None


def load_library(path: Optional[str] = None) -> ctypes.CDLL:
    """Load libamca3d.so (built by ``amca3d_gb300.build``). Raises if absent."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = path or LIB_PATH
    if not os.path.exists(p):
        raise FileNotFoundError(f"{p} is missing: build it with `python -m amca3d_gb300.build` "
                                f"(no CPU fallback exists)")
    lib = ctypes.CDLL(p)
    vp, cp, i, i64 = ctypes.c_void_p, ctypes.c_char_p, ctypes.c_int, ctypes.c_int64
    lib.amca_create.argtypes = [cp, ctypes.POINTER(_Opts), ctypes.POINTER(vp)]
    lib.amca_get_grid.argtypes = [vp, ctypes.POINTER(ctypes.c_int32), ctypes.POINTER(ctypes.c_double),
                                  ctypes.POINTER(ctypes.c_double)]
    lib.amca_prepare.argtypes = [vp]
    lib.amca_get_sites.argtypes = [vp, vp, vp, ctypes.c_size_t, ctypes.POINTER(ctypes.c_size_t)]
    lib.amca_initialize.argtypes = [vp]
    lib.amca_step.argtypes = [vp, ctypes.POINTER(ctypes.c_double)]
    lib.amca_run.argtypes = [vp, i]
    lib.amca_get_field.argtypes = [vp, i, vp, ctypes.c_size_t]
    lib.amca_get_orientations.argtypes = [vp, ctypes.POINTER(ctypes.c_double), ctypes.c_size_t,
                                          ctypes.POINTER(ctypes.c_size_t), i]
    lib.amca_write_outputs.argtypes = [vp]
    lib.amca_get_stats.argtypes = [vp, ctypes.POINTER(Stats)]
    lib.amca_envelope_eval.argtypes = [i, ctypes.c_size_t, vp, vp, vp, ctypes.c_double, vp, vp, vp, vp]
    lib.amca_envelope_eval.restype = i
    lib.amca_selftest_barrier.argtypes = [i, i, i, ctypes.c_int64, ctypes.c_int32, vp, vp]
    lib.amca_selftest_barrier.restype = i
    lib.amca_release_cached_memory.argtypes = [i]
    lib.amca_release_cached_memory.restype = i
    lib.amca_final_grain_count.argtypes = [vp, ctypes.POINTER(ctypes.c_int32)]
    lib.amca_final_grain_count.restype = i
    lib.amca_reset.argtypes = [vp]
    lib.amca_reset.restype = i
    lib.amca_host_alloc.argtypes = [ctypes.c_size_t, ctypes.POINTER(vp)]
    lib.amca_host_alloc.restype = i
    lib.amca_host_free.argtypes = [vp]
    lib.amca_host_free.restype = i
    lib.amca_plain_run_noalloc.argtypes = [i, ctypes.POINTER(PlainParams), vp, vp, ctypes.c_int64, vp, vp, i, vp,
                                           ctypes.POINTER(PlainResult), ctypes.c_char_p, ctypes.c_size_t]
    lib.amca_plain_run_noalloc.restype = i
    lib.amca_set_fe_frames.argtypes = [vp, ctypes.POINTER(ctypes.c_int32), vp, ctypes.c_int32, vp, vp]
    lib.amca_set_fe_frames.restype = i
    lib.amca_set_rosenthal_frames.argtypes = [vp, ctypes.POINTER(Rosenthal)]
    lib.amca_set_rosenthal_frames.restype = i
    lib.amca_set_microstructure.argtypes = [vp, vp, vp, vp, vp, i64, vp, i64, vp, vp, i64]
    lib.amca_set_microstructure.restype = i
    lib.amca_batch_create.argtypes = [ctypes.POINTER(vp), i, i, ctypes.POINTER(vp)]
    lib.amca_batch_create.restype = i
    lib.amca_batch_run.argtypes = [vp, ctypes.POINTER(ctypes.c_double)]
    lib.amca_batch_run.restype = i
    lib.amca_batch_tune.argtypes = [vp, i, ctypes.POINTER(ctypes.c_int)]
    lib.amca_batch_tune.restype = i
    lib.amca_batch_set_layout.argtypes = [vp, i, vp, vp, vp, vp]
    lib.amca_batch_set_layout.restype = i
    lib.amca_batch_get_layout.argtypes = [vp, i, vp, vp, vp, vp, ctypes.POINTER(ctypes.c_int)]
    lib.amca_batch_get_layout.restype = i
    lib.amca_batch_get_stats.argtypes = [vp, ctypes.POINTER(BatchStats)]
    lib.amca_batch_get_stats.restype = i
    lib.amca_batch_last_error.argtypes = [vp]
    lib.amca_batch_last_error.restype = cp
    lib.amca_batch_destroy.argtypes = [vp]
    lib.amca_batch_destroy.restype = None
    lib.amca_last_error.argtypes = [vp]
    lib.amca_last_error.restype = cp
    lib.amca_destroy.argtypes = [vp]
    lib.amca_destroy.restype = None
    lib.amca_step_coupled.argtypes = [vp, ctypes.c_double, ctypes.POINTER(ctypes.c_double)]
    lib.amca_step_coupled.restype = i
    lib.amca_run_until.argtypes = [vp, ctypes.c_double]
    lib.amca_run_until.restype = i
    lib.amca_set_nodal_temperatures.argtypes = [vp, vp, i64]
    lib.amca_set_nodal_temperatures.restype = i
    lib.amca_set_scan_frames.argtypes = [vp, ctypes.POINTER(Scan)]
    lib.amca_set_scan_frames.restype = i
    lib.amca_set_thermal_frames.argtypes = [vp, vp, ctypes.POINTER(Scan), ctypes.c_double, ctypes.c_double,
                                            ctypes.c_double]
    lib.amca_set_thermal_frames.restype = i
    lib.amca_get_frame_stats.argtypes = [vp, vp]
    lib.amca_get_frame_stats.restype = i
    lib.amca_thermal_create.argtypes = [i, ctypes.POINTER(ThermalSpec), ctypes.POINTER(vp)]
    lib.amca_thermal_create.restype = i
    lib.amca_thermal_train.argtypes = [vp, i64, i, i, ctypes.c_double, ctypes.c_double,
                                       ctypes.POINTER(ThermalTrainStats)]
    lib.amca_thermal_train.restype = i
    lib.amca_thermal_eval.argtypes = [vp, vp, i64, vp, vp]
    lib.amca_thermal_eval.restype = i
    lib.amca_thermal_gradients.argtypes = [vp, vp, vp, i64, vp, vp]
    lib.amca_thermal_gradients.restype = i
    lib.amca_thermal_param_count.argtypes = []
    lib.amca_thermal_param_count.restype = i64
    lib.amca_thermal_get_params.argtypes = [vp, vp]
    lib.amca_thermal_get_params.restype = i
    lib.amca_thermal_set_params.argtypes = [vp, vp]
    lib.amca_thermal_set_params.restype = i
    lib.amca_thermal_get_encoding.argtypes = [vp, vp, vp, vp, vp, vp, vp]
    lib.amca_thermal_get_encoding.restype = i
    lib.amca_thermal_frames.argtypes = [vp, ctypes.POINTER(Scan), ctypes.c_int32, ctypes.c_int32, ctypes.c_double,
                                        ctypes.c_double, ctypes.c_double, vp, vp, vp]
    lib.amca_thermal_frames.restype = i
    lib.amca_thermal_last_error.argtypes = [vp]
    lib.amca_thermal_last_error.restype = cp
    lib.amca_thermal_destroy.argtypes = [vp]
    lib.amca_thermal_destroy.restype = None
    for name in ("amca_create", "amca_get_grid", "amca_prepare", "amca_get_sites", "amca_initialize", "amca_step",
                 "amca_run", "amca_get_field", "amca_get_orientations", "amca_write_outputs", "amca_get_stats"):
        getattr(lib, name).restype = i
    if path is None:
        _lib = lib
    return lib


class PinnedBuffer:
    """Page-locked host array (cudaMallocHost) for fast field copies."""

    def __init__(self, n: int, dtype=np.int32):
        self._lib = load_library()
        self._p = ctypes.c_void_p()
        nbytes = int(n) * np.dtype(dtype).itemsize
        rc = self._lib.amca_host_alloc(nbytes, ctypes.byref(self._p))
        if rc != AMCA_OK:
            raise AmcaError(rc, self._lib.amca_last_error(None).decode())
        buf = (ctypes.c_char * nbytes).from_address(self._p.value)
        self.array = np.frombuffer(buf, dtype=dtype, count=int(n))

    def free(self) -> None:
        if self._p:
            self.array = None
            self._lib.amca_host_free(self._p)
            self._p = ctypes.c_void_p()

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


def envelope_eval(l2g: np.ndarray, gc: np.ndarray, length: np.ndarray, h: float, trunc: np.ndarray,
                  device: int = 0):
    """Run the envelope arithmetic (Octahedron::cell_is_captured / capture_cell)
    on the GPU for independent pairs. Returns (captured_fp64, captured_fast, info)."""
    lib = load_library()
    n = len(length)
    l2g = np.ascontiguousarray(l2g, np.float64).reshape(n, 9)
    gc = np.ascontiguousarray(gc, np.float64).reshape(n, 3)
    length = np.ascontiguousarray(length, np.float64)
    trunc = np.ascontiguousarray(trunc, np.float64)
    cap = np.empty(n, np.int32)
    fast = np.empty(n, np.int32)
    info = np.empty((n, 4), np.float64)
    ptr = lambda a: a.ctypes.data_as(ctypes.c_void_p)  # noqa: E731
    rc = lib.amca_envelope_eval(device, n, ptr(l2g), ptr(gc), ptr(length), h, ptr(trunc), ptr(cap), ptr(fast),
                                ptr(info))
    if rc != AMCA_OK:
        raise AmcaError(rc, lib.amca_last_error(None).decode())
    return cap, fast, info


def release_cached_memory(device: int = -1) -> None:
    """Free the device arena kept from destroyed realms (amca_release_cached_memory)."""
    lib = load_library()
    rc = lib.amca_release_cached_memory(device)
    if rc != AMCA_OK:
        raise AmcaError(rc, lib.amca_last_error(None).decode())


def selftest_barrier(blocks: int, parties: int, wait_ns: int, preset_error: int = 0, device: int = 0):
    """Run the step kernels' bounded grid barrier once on `blocks` blocks
    expecting `parties` arrivals (amca_selftest_barrier). Returns (error word
    afterwards, per-block verdicts: 1 = the barrier returned success)."""
    lib = load_library()
    err = ctypes.c_int32(0)
    verdicts = np.zeros(blocks, np.int32)
    rc = lib.amca_selftest_barrier(device, blocks, parties, int(wait_ns), int(preset_error), ctypes.byref(err),
                                   verdicts.ctypes.data_as(ctypes.c_void_p))
    if rc != AMCA_OK:
        raise AmcaError(rc, lib.amca_last_error(None).decode())
    return int(err.value), verdicts


class CellularAutomataRealm:
    """One AMCA3D CA realm on one GPU, read from a YAML deck."""

    def __init__(self, deck: str, seed: int = 0, device: int = 0, write_outputs: bool = False,
                 workdir: Optional[str] = None):
        self._lib = load_library()
        self._h = ctypes.c_void_p()
        self._workdir = workdir.encode() if workdir else None
        opts = _Opts(device, seed, 1 if write_outputs else 0, self._workdir)
        rc = self._lib.amca_create(deck.encode(), ctypes.byref(opts), ctypes.byref(self._h))
        if rc != AMCA_OK:
            raise AmcaError(rc, self._lib.amca_last_error(None).decode())
        cells = (ctypes.c_int32 * 3)()
        origin = (ctypes.c_double * 3)()
        h = ctypes.c_double()
        self._check(self._lib.amca_get_grid(self._h, cells, origin, ctypes.byref(h)))
        self.cells = tuple(int(c) for c in cells)
        self.origin = tuple(float(o) for o in origin)
        self.cell_size = h.value
        self._ghost_cells = (self.cells[0] + 2) * (self.cells[1] + 2) * (self.cells[2] + 2)

    def _check(self, rc: int) -> None:
        if rc != AMCA_OK:
            raise AmcaError(rc, self._lib.amca_last_error(self._h).decode())

    def prepare(self) -> None:
        """Host half of initialize (sites, orientation stream); needs no GPU."""
        self._check(self._lib.amca_prepare(self._h))

    def sites(self):
        """(cell ids, critical undercoolings) of the nucleation sites after prepare()."""
        n = ctypes.c_size_t()
        self._check(self._lib.amca_get_sites(self._h, None, None, 0, ctypes.byref(n)))
        cells = np.empty(n.value, np.int32)
        dtc = np.empty(n.value, np.float64)
        self._check(self._lib.amca_get_sites(self._h, cells.ctypes.data_as(ctypes.c_void_p),
                                             dtc.ctypes.data_as(ctypes.c_void_p), n.value, ctypes.byref(n)))
        return cells, dtc

    def initialize(self) -> None:
        self._check(self._lib.amca_initialize(self._h))

    def single_integration_step(self) -> float:
        dt = ctypes.c_double()
        self._check(self._lib.amca_step(self._h, ctypes.byref(dt)))
        return dt.value

    def run(self, max_steps: int = -1) -> None:
        self._check(self._lib.amca_run(self._h, int(max_steps)))

    def step_coupled(self, dt_cap: float) -> float:
        """One step with dt also bounded by dt_cap (setup_time_step_for_coupling)."""
        dt = ctypes.c_double()
        self._check(self._lib.amca_step_coupled(self._h, float(dt_cap), ctypes.byref(dt)))
        return dt.value

    def run_until(self, t_end: float) -> None:
        """Steps while time < t_end."""
        self._check(self._lib.amca_run_until(self._h, float(t_end)))

    def set_nodal_temperatures(self, theta: np.ndarray) -> None:
        """FE-coupled decks: node temperatures the next step interpolates (an
        external FE solver's thetaArray_); the realm stops replaying frames."""
        t = np.ascontiguousarray(theta, np.float64)
        self._check(self._lib.amca_set_nodal_temperatures(self._h, t.ctypes.data_as(ctypes.c_void_p), t.size))

    time_integration = run

    def stats(self) -> dict:
        s = Stats()
        self._check(self._lib.amca_get_stats(self._h, ctypes.byref(s)))
        return s.as_dict()

    def set_fe_frames(self, nodes, coords: np.ndarray, times: np.ndarray, theta: np.ndarray) -> None:
        """FE-coupled decks: frames from memory in the file's units (replaces the
        deck's frame file)."""
        nn = (ctypes.c_int32 * 3)(*[int(v) for v in nodes])
        coords = np.ascontiguousarray(coords, np.float64)
        times = np.ascontiguousarray(times, np.float64)
        theta = np.ascontiguousarray(theta, np.float64)
        ptr = lambda a: a.ctypes.data_as(ctypes.c_void_p)  # noqa: E731
        self._check(self._lib.amca_set_fe_frames(self._h, nn, ptr(coords), len(times), ptr(times), ptr(theta)))

    def set_microstructure(self, grain, orient, euler, grain_cell, grain_orient, melted=None, dtc=None,
                           expected: int = 0) -> None:
        """FE-coupled decks: restart microstructure from memory (the content of
        grainInfo<rank>.txt); replaces the deck's random or file microstructure."""
        grain = np.ascontiguousarray(grain, np.int32)
        orient = np.ascontiguousarray(orient, np.int32)
        euler = np.ascontiguousarray(euler, np.float64).reshape(-1, 3)
        grain_cell = np.ascontiguousarray(grain_cell, np.int32)
        grain_orient = np.ascontiguousarray(grain_orient, np.int32)
        melted = None if melted is None else np.ascontiguousarray(melted, np.uint8)
        dtc = None if dtc is None else np.ascontiguousarray(dtc, np.float64)
        ptr = lambda a: None if a is None else a.ctypes.data_as(ctypes.c_void_p)  # noqa: E731
        self._check(self._lib.amca_set_microstructure(self._h, ptr(grain), ptr(orient), ptr(melted), ptr(dtc),
                                                      len(euler), ptr(euler), len(grain_cell), ptr(grain_cell),
                                                      ptr(grain_orient), int(expected)))

    def set_rosenthal_frames(self, **kw) -> None:
        """FE-coupled decks: frames generated on the GPU (fields of amca_rosenthal)."""
        r = Rosenthal()
        for k, v in kw.items():
            if k in ("origin", "nodes"):
                for a in range(3):
                    getattr(r, k)[a] = v[a]
            else:
                setattr(r, k, v)
        self._check(self._lib.amca_set_rosenthal_frames(self._h, ctypes.byref(r)))

    def set_scan_frames(self, **kw) -> None:
        """FE-coupled decks: frames of a raster scan's FE field (fields of
        amca_scan), produced on the GPU a window at a time."""
        self._scan = Scan.of(**kw)
        self._check(self._lib.amca_set_scan_frames(self._h, ctypes.byref(self._scan)))

    def set_thermal_frames(self, model: "ThermalModel", t_liq: float, band: float, thresh: float, **kw) -> None:
        """FE-coupled decks: frames of a raster scan from a trained thermal
        model, with the FE field where the model's error estimate exceeds
        thresh within band of t_liq (K). The model must outlive the realm."""
        self._scan = Scan.of(**kw)
        self._model = model
        self._check(self._lib.amca_set_thermal_frames(self._h, model.handle, ctypes.byref(self._scan), float(t_liq),
                                                      float(band), float(thresh)))

    def frame_stats(self) -> dict:
        out = np.zeros(5, np.int64)
        self._check(self._lib.amca_get_frame_stats(self._h, out.ctypes.data_as(ctypes.c_void_p)))
        return dict(frames=int(out[0]), fills=int(out[1]), model_nodes=int(out[2]), near_liquidus=int(out[3]),
                    fallbacks=int(out[4]))

    def field(self, name: str = "orientation_id", out: Optional[np.ndarray] = None) -> np.ndarray:
        fid = FIELD_IDS[name]
        n = self.cells_with_ghosts
        dtype = FIELD_DTYPES[name]
        if out is None:
            out = np.empty(n, dtype=dtype)
        assert out.dtype == dtype and out.size == n and out.flags.c_contiguous
        self._check(self._lib.amca_get_field(self._h, fid, out.ctypes.data_as(ctypes.c_void_p), out.nbytes))
        return out

    def orientations(self, all: bool = False) -> np.ndarray:
        """Euler angles of the orientations created so far (all=True: the whole
        pre-drawn stream, one per site)."""
        n = ctypes.c_size_t()
        self._check(self._lib.amca_get_orientations(self._h, None, 0, ctypes.byref(n), int(all)))
        e = np.empty((n.value, 3), np.float64)
        self._check(self._lib.amca_get_orientations(self._h, e.ctypes.data_as(ctypes.POINTER(ctypes.c_double)),
                                                    n.value, ctypes.byref(n), int(all)))
        return e

    def write_outputs(self) -> None:
        self._check(self._lib.amca_write_outputs(self._h))

    def reset(self) -> None:
        """Back to the state right after initialize(), tables kept in HBM."""
        self._check(self._lib.amca_reset(self._h))

    def final_grain_count(self) -> int:
        n = ctypes.c_int32()
        self._check(self._lib.amca_final_grain_count(self._h, ctypes.byref(n)))
        return n.value

    @property
    def cells_with_ghosts(self) -> int:
        return self._ghost_cells

    def close(self) -> None:
        if self._h:
            self._lib.amca_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()


class Batch:
    """Many initialized plain realms run in one cooperative launch
    (amca_batch_*): teams of blocks pull realms from a queue; every realm's
    result is the one it gives when run alone. The realms must stay open
    while the batch exists."""

    def __init__(self, realms, team_size: int = 0):
        self._lib = load_library()
        self.realms = list(realms)
        arr = (ctypes.c_void_p * max(len(self.realms), 1))(*[r._h.value for r in self.realms])
        self._b = ctypes.c_void_p()
        rc = self._lib.amca_batch_create(arr, len(self.realms), int(team_size), ctypes.byref(self._b))
        if rc != AMCA_OK:
            raise AmcaError(rc, self._lib.amca_batch_last_error(None).decode())

    def _check(self, rc: int) -> None:
        if rc != AMCA_OK:
            raise AmcaError(rc, self._lib.amca_batch_last_error(self._b).decode())

    def run(self) -> float:
        """Every realm from its initial state to its end; returns device ms."""
        ms = ctypes.c_double()
        self._check(self._lib.amca_batch_run(self._b, ctypes.byref(ms)))
        return ms.value

    def set_layout(self, team_size, teams, realm_class, queue_order=None) -> None:
        """Class c = teams[c] teams of team_size[c] blocks; realm r runs in
        class realm_class[r]; queue_order (optional) orders each class's
        queue."""
        vp = ctypes.c_void_p
        ts = np.ascontiguousarray(team_size, np.int32)
        tn = np.ascontiguousarray(teams, np.int32)
        rc = np.ascontiguousarray(realm_class, np.int32)
        if len(ts) != len(tn) or len(rc) != len(self.realms):
            raise ValueError("team_size and teams need one entry per class, realm_class one per realm")
        qo = None if queue_order is None else np.ascontiguousarray(queue_order, np.int32)
        if qo is not None and len(qo) != len(self.realms):
            raise ValueError("queue_order needs one entry per realm")
        self._check(self._lib.amca_batch_set_layout(self._b, len(ts), ts.ctypes.data_as(vp), tn.ctypes.data_as(vp),
                                                    rc.ctypes.data_as(vp),
                                                    None if qo is None else qo.ctypes.data_as(vp)))

    def layout(self):
        """(team_size, teams, realm_class, queue_order) of the current layout."""
        vp = ctypes.c_void_p
        nc = ctypes.c_int()
        self._check(self._lib.amca_batch_get_layout(self._b, 0, None, None, None, None, ctypes.byref(nc)))
        ts = np.zeros(nc.value, np.int32)
        tn = np.zeros(nc.value, np.int32)
        rc = np.zeros(len(self.realms), np.int32)
        qo = np.zeros(len(self.realms), np.int32)
        self._check(self._lib.amca_batch_get_layout(self._b, nc.value, ts.ctypes.data_as(vp), tn.ctypes.data_as(vp),
                                                    rc.ctypes.data_as(vp), qo.ctypes.data_as(vp), ctypes.byref(nc)))
        return ts, tn, rc, qo

    def tune(self, repeats: int = 1) -> int:
        t = ctypes.c_int()
        self._check(self._lib.amca_batch_tune(self._b, int(repeats), ctypes.byref(t)))
        return t.value

    def stats(self) -> dict:
        s = BatchStats()
        self._check(self._lib.amca_batch_get_stats(self._b, ctypes.byref(s)))
        return s.as_dict()

    def close(self) -> None:
        if self._b:
            self._lib.amca_batch_destroy(self._b)
            self._b = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()


class ThermalModel:
    """The learned thermal model (amca_thermal_* of include/amca3d.h): a
    Fourier-feature MLP trained on the GPU by the library's tensor-core
    kernels to stand in for the FE nodal temperatures of a scanning laser."""

    def __init__(self, device: int = 0, **spec):
        self._lib = load_library()
        s = ThermalSpec()
        for k, v in spec.items():
            if k in ("window_lo", "window_hi", "near_lo", "near_hi"):
                for a in range(3):
                    getattr(s, k)[a] = v[a]
            else:
                setattr(s, k, v)
        self.spec = spec
        self._h = ctypes.c_void_p()
        rc = self._lib.amca_thermal_create(int(device), ctypes.byref(s), ctypes.byref(self._h))
        if rc != AMCA_OK:
            raise AmcaError(rc, "amca_thermal_create failed (check the spec ranges)")

    @property
    def handle(self) -> ctypes.c_void_p:
        return self._h

    def _check(self, rc: int) -> None:
        if rc != AMCA_OK:
            raise AmcaError(rc, self._lib.amca_thermal_last_error(self._h).decode())

    @staticmethod
    def param_count() -> int:
        return int(load_library().amca_thermal_param_count())

    def train(self, samples: int, steps: int, batch: int, lr_max: float = 1e-3, lr_min: float = 1e-5) -> dict:
        st = ThermalTrainStats()
        self._check(self._lib.amca_thermal_train(self._h, int(samples), int(steps), int(batch), float(lr_max),
                                                 float(lr_min), ctypes.byref(st)))
        return {k: getattr(st, k) for k, _ in st._fields_}

    def eval(self, raw: np.ndarray):
        """(T, error estimate) in K for raw inputs [n x 5]."""
        raw = np.ascontiguousarray(raw, np.float32).reshape(-1, 5)
        n = raw.shape[0]
        T = np.zeros(n, np.float32)
        e = np.zeros(n, np.float32)
        vp = ctypes.c_void_p
        self._check(self._lib.amca_thermal_eval(self._h, raw.ctypes.data_as(vp), n, T.ctypes.data_as(vp),
                                                e.ctypes.data_as(vp)))
        return T, e

    def gradients(self, raw: np.ndarray, target: np.ndarray):
        """(gradient vector, [n x 2] outputs mu, s) of one batch; no update."""
        raw = np.ascontiguousarray(raw, np.float32).reshape(-1, 5)
        y = np.ascontiguousarray(target, np.float32)
        g = np.zeros(self.param_count(), np.float32)
        pred = np.zeros((raw.shape[0], 2), np.float32)
        vp = ctypes.c_void_p
        self._check(self._lib.amca_thermal_gradients(self._h, raw.ctypes.data_as(vp), y.ctypes.data_as(vp),
                                                     raw.shape[0], g.ctypes.data_as(vp), pred.ctypes.data_as(vp)))
        return g, pred

    def params(self) -> np.ndarray:
        p = np.zeros(self.param_count(), np.float32)
        self._check(self._lib.amca_thermal_get_params(self._h, p.ctypes.data_as(ctypes.c_void_p)))
        return p

    def set_params(self, p: np.ndarray) -> None:
        p = np.ascontiguousarray(p, np.float32)
        if p.size != self.param_count():
            raise ValueError("wrong parameter count")
        self._check(self._lib.amca_thermal_set_params(self._h, p.ctypes.data_as(ctypes.c_void_p)))

    def encoding(self) -> dict:
        f = np.zeros(64 * 5, np.float32)
        sh = np.zeros(5, np.float32)
        sc = np.zeros(5, np.float32)
        ts, tsc, lo = ctypes.c_float(), ctypes.c_float(), ctypes.c_int32()
        vp = ctypes.c_void_p
        self._check(self._lib.amca_thermal_get_encoding(self._h, f.ctypes.data_as(vp), sh.ctypes.data_as(vp),
                                                        sc.ctypes.data_as(vp), ctypes.byref(ts), ctypes.byref(tsc),
                                                        ctypes.byref(lo)))
        return dict(fourier=f.reshape(64, 5), in_shift=sh, in_scale=sc, t_shift=ts.value, t_scale=tsc.value,
                    log_output=int(lo.value))

    def frames(self, scan: Scan, f0: int, nf: int, t_liq: float, band: float, thresh: float, with_fe: bool = False):
        """(model frames [nf x nodes], FE frames or None, counts: evaluated, near the liquidus, fallbacks)."""
        nn = scan.nodes[0] * scan.nodes[1] * scan.nodes[2]
        out = np.zeros((nf, nn), np.float64)
        fe = np.zeros((nf, nn), np.float64) if with_fe else None
        counts = np.zeros(3, np.int64)
        vp = ctypes.c_void_p
        self._check(self._lib.amca_thermal_frames(self._h, ctypes.byref(scan), int(f0), int(nf), float(t_liq),
                                                  float(band), float(thresh), out.ctypes.data_as(vp),
                                                  None if fe is None else fe.ctypes.data_as(vp),
                                                  counts.ctypes.data_as(vp)))
        return out, fe, counts

    def close(self) -> None:
        if self._h:
            self._lib.amca_thermal_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
