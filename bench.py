"""Benchmark: plain CA timestep, uniform cooling at 320^3 (32.8M cells);
with --workload pbf_500 the FE-coupled remelting realm on a laser track
(500 x 250 x 100 cells, Rosenthal frames, columnar baseplate); with
--workload batched_64 64 independent plain instances (edges 32..128) in one
graph-replayed launch, beside the same instances as 64 sequential launches;
with --workload thermal_1024 the 134M-cell 5-track raster on frames of the
FE field and on frames of the learned thermal model (trained first).

One bench step = one full run of the deck from its initial state to its end
(full solidification, or the end of the frames), every CA step of it, on one
GPU; cell-updates/s = interior cells x CA steps / time. The default line
(uniform_320, one GPU) also carries the pbf_500 and batched_64 results under
those keys, each measured with its own warm-up, timed runs, clocks and
roofline (--no-extra leaves them out).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                  [--workload uniform_320|pbf_500|batched_64|thermal_1024]

ours (default): the CUDA path. `value` is device time (CUDA events around
  the persistent step kernel on its stream) with the realm's tables resident
  in HBM; `e2e` is the same metric through the public C ABI per step
  (amca_create -> amca_initialize (host sites + H2D) -> amca_run ->
  amca_get_field into pinned host memory -> amca_destroy), wall clock.
reference: the CPU implementation of the path (the C restatement of the
  reference, one process per host core, each on a bounded sample of the
  workload), same metric.
For N > 1 (torchrun) each rank of uniform_320 and pbf_500 runs an independent
replica (a single domain does not shard under bit-exactness); batched_64
partitions its 64 instances over the ranks (longest first, no collective on
the data path; the per-instance field digests are gathered and checked
against the instances' reference runs). The value is the sum of cell updates
over ranks divided by the slowest rank's time.
"""
from __future__ import annotations

import argparse
import dataclasses
import json
import multiprocessing as mp
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

from amca3d_gb300 import decks  # noqa: E402

METRIC = "cell-updates/s on 1 GB300, plain vs surrogate/batched, at matched grain stats"
UNIT = "cell-updates/s"
# AMCA_PHASE_DETAIL=1 makes the kernels also gather the slowest block's busy
# time per phase (a global load per block and barrier); reported only then
PHASE_DETAIL = os.environ.get("AMCA_PHASE_DETAIL", "0") not in ("", "0")


def workload():
    return decks.config_uniform_320()


def sample_case(n: int):
    """The workload's physics on an n^3 block: same cell size, cooling and
    site densities (surface sites scale with area, bulk with volume)."""
    c = workload()
    s = n / 320
    return dataclasses.replace(
        c, name=f"uniform_{n}", cells=(n, n, n),
        surface=(decks.surface_density_for_sites(4000 * s * s, (n, n, n), c.cell_size), 2.0, 0.5),
        bulk=(decks.bulk_density_for_sites(20000 * s ** 3, (n, n, n), c.cell_size), 3.0, 1.0))


# ----------------------------------------------------------------------------
# distributed helpers (gloo: only a barrier and a max/sum of scalars)
# ----------------------------------------------------------------------------
class Dist:
    def __init__(self):
        self.world = int(os.environ.get("WORLD_SIZE", "1"))
        self.rank = int(os.environ.get("RANK", "0"))
        self.local_rank = int(os.environ.get("LOCAL_RANK", "0"))
        self.pg = None
        if self.world > 1:
            import torch.distributed as dist

            dist.init_process_group("gloo")
            self.pg = dist

    def barrier(self):
        if self.pg:
            self.pg.barrier()

    def reduce(self, x: float, op: str) -> float:
        if not self.pg:
            return x
        import torch

        t = torch.tensor([x], dtype=torch.float64)
        self.pg.all_reduce(t, op=self.pg.ReduceOp.MAX if op == "max" else self.pg.ReduceOp.SUM)
        return float(t.item())

    def gather(self, obj) -> list:
        """Every rank's object, in rank order, on every rank."""
        if not self.pg:
            return [obj]
        out = [None] * self.world
        self.pg.all_gather_object(out, obj)
        return out

    def close(self):
        if self.pg:
            self.pg.destroy_process_group()


# ----------------------------------------------------------------------------
# clocks during the timed region
# ----------------------------------------------------------------------------
class ClockSampler:
    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.QUERY}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except (OSError, FileNotFoundError):
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self) -> dict:
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.thread.join(timeout=2)
        sm, smax, power, reasons = [], [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax.append(float(f[2]))
                power.append(float(f[3]))
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(smax), "reasons": sorted(reasons),
                "samples": len(sm), "power_w_max": max(power)}


# ----------------------------------------------------------------------------
# grain statistics (matched-stats columns of the metric)
# ----------------------------------------------------------------------------
def grain_stats(orient: np.ndarray, cells, euler: np.ndarray) -> dict:
    nx, ny, nz = cells
    inner = orient.reshape(nz + 2, ny + 2, nx + 2)[1:-1, 1:-1, 1:-1].ravel()
    ids, counts = np.unique(inner[inner >= 0], return_counts=True)
    # <100> || z within 15 deg: max over crystal axes of |z-component| of the
    # local->global matrix column (Bunge ZXZ, Octahedron.cpp:282-310)
    a, b, g = euler[ids, 0], euler[ids, 1], euler[ids, 2]
    zcol = np.stack([np.sin(b) * np.sin(g), np.sin(b) * np.cos(g), np.cos(b)], 1)
    aligned = np.abs(zcol).max(1) >= np.cos(np.deg2rad(15.0))
    return {"grains": int(len(ids)), "mean_grain_cells": float(counts.mean()) if len(ids) else 0.0,
            "texture_100_z_15deg": float(counts[aligned].sum() / counts.sum()) if len(ids) else 0.0}


# ----------------------------------------------------------------------------
# CPU oracle runs (bounded samples)
# ----------------------------------------------------------------------------
def _oracle_sample(n: int) -> tuple:
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import amca_oracle

    case = sample_case(n)
    t = time.perf_counter()
    r = amca_oracle.run_plain(case, fields=False)
    el = time.perf_counter() - t
    return case.n_interior * r["steps"], el, r["steps"]


def cpu_baseline(n: int = 128) -> dict:
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import amca_oracle

    amca_oracle.build()
    upd, el, steps = _oracle_sample(n)
    return {"value": upd / el, "unit": UNIT, "cores": 1, "kind": "port",
            "sample": f"C restatement of the reference, one core: the workload's physics on a {n}^3 block "
                      f"(same h, cooling, site densities), {steps} CA steps to full solidification, {el:.1f} s"}


def run_reference_arm(args, dist: Dist):
    if dist.rank != 0:
        return
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import amca_oracle

    amca_oracle.build()
    cores = os.cpu_count() or 1
    n = args.ref_sample
    ctx = mp.get_context("spawn")
    times, updates = [], []
    with ctx.Pool(cores) as pool:
        for it in range(args.warmup + args.steps):
            t = time.perf_counter()
            res = pool.map(_oracle_sample, [n] * cores)
            el = time.perf_counter() - t
            if it >= args.warmup:
                times.append(el)
                updates.append(sum(r[0] for r in res))
    value = sum(updates) / sum(times)
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * sum(times) / len(times),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": config_block(None),
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port",
                         "sample": f"{cores} concurrent single-core runs of the C restatement of the reference "
                                   f"(the reference is sequential per MPI rank and mpirun is not used here), "
                                   f"each the workload's physics on a {n}^3 block run to full solidification"},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def config_block(stats, case=None) -> dict:
    c = case or workload()
    if c.cells == (320, 320, 320):
        text = ("uniform_320: plain CA, uniform cooling, 320^3 cells of 2 um (32.8M), t_dot = -50 K/s, "
                "~20k bulk Gaussian sites (3 K, 1 K) + ~4k surface sites (2 K, 0.5 K), KGT a1=-0.544e-4 "
                "a2=2.03e-4, seed 1, every CA step to full solidification")
    else:
        text = f"{c.name}: the uniform_320 physics on a {c.cells[0]}^3 block (profiling case, not the workload)"
    cfg = {"workload": text, "cells": c.n_interior, "seed": c.seed, "envelope_arith": "fp64", "grain_ids": "int32",
           "l2": "inputs larger than L2: orientation field 134 MB + envelope table 1.7 GB per run"}
    if stats:
        cfg.update(stats)
    return cfg


def load_traffic(name: str = "ca_persistent_uniform_320.json"):
    p = os.path.join(ROOT, "profiles", name)
    if os.path.exists(p):
        try:
            return json.load(open(p)).get("dram_bytes_per_launch")
        except (OSError, ValueError):
            return None
    return None


def measured_peak():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def run_ours(args, dist: Dist):
    import amca3d_gb300 as A

    dev = dist.local_rank
    case = workload() if args.cells == 320 else sample_case(args.cells)
    deck = case.to_yaml()
    realm = A.CellularAutomataRealm(deck, seed=case.seed, device=dev)
    realm.initialize()
    for _ in range(args.warmup):
        realm.reset()
        realm.run()
    clocks = ClockSampler(dev)
    dist.barrier()
    clocks.start()
    device_ms, updates, ca_steps, alg_bytes, launches = [], [], [], [], 0
    t0 = time.perf_counter()
    for _ in range(args.steps):
        realm.reset()
        realm.run()
        st = realm.stats()
        device_ms.append(st["kernel_ms"])
        updates.append(st["cells"] * st["step"])
        ca_steps.append(st["step"])
        alg_bytes.append(st["algorithmic_bytes"])
        launches += st["launches"] + 1  # the persistent kernel launches + the field reset kernel
    wall = time.perf_counter() - t0
    dist.barrier()
    clk = clocks.stop()
    st = realm.stats()
    orient = realm.field("orientation_id")
    gstats = grain_stats(orient, case.cells, realm.orientations())
    realm.close()

    # end to end through the public API, host buffers, per step
    pinned = A.PinnedBuffer(case.n_ghost, np.int32)
    e2e_t, e2e_upd, h2d, d2h = [], [], [], []
    for it in range(args.warmup + args.steps):
        t = time.perf_counter()
        r = A.CellularAutomataRealm(deck, seed=case.seed, device=dev)
        r.initialize()
        r.run()
        r.field("orientation_id", out=pinned.array)
        s = r.stats()
        r.close()
        el = time.perf_counter() - t
        if it >= args.warmup:
            e2e_t.append(el)
            e2e_upd.append(s["cells"] * s["step"])
            h2d.append(s["h2d_bytes"])
            d2h.append(s["d2h_bytes"])
    same = bool(np.array_equal(pinned.array, orient))
    pinned.free()

    t_dev = dist.reduce(sum(device_ms) / 1e3, "max")
    upd_total = dist.reduce(float(sum(updates)), "sum")
    e2e_time = dist.reduce(sum(e2e_t), "max")
    e2e_total = dist.reduce(float(sum(e2e_upd)), "sum")
    if dist.rank != 0:
        return
    peak, peak_kind = measured_peak()
    achieved = (sum(alg_bytes) / len(alg_bytes)) / (sum(device_ms) / len(device_ms) / 1e3) / 1e9
    traffic = load_traffic()
    line = {
        "metric": METRIC, "value": upd_total / t_dev, "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": sum(device_ms) / len(device_ms), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": config_block({"ca_steps_per_run": ca_steps[-1], "envelopes": st["grains"], **gstats,
                                "generations_per_run": st["generations"], "tests_per_run": st["tests"],
                                "phase_ms_nucleation_claim_resolve_end": [round(x, 3) for x in st["phase_ms"][:4]],
                                "phase_ms_claim_gen0": round(st["phase_ms"][4], 3),
                                "busy_ms_mean_claim_resolve": [round(st["phase_ms"][5], 3),
                                                               round(st["phase_ms"][7], 3)],
                                **({"busy_ms_slowest_claim_resolve": [round(st["phase_ms"][6], 3),
                                                                      round(st["phase_ms"][8], 3)],
                                    "busy_ms_slowest_nucleation_wake": round(st["detail_ms"][3], 3)}
                                   if PHASE_DETAIL else {}),
                                "fp64_tests_per_run": st["tests_fp64"],
                                "busy_ms_mean_nucleation_wake_compaction": [round(x, 3) for x in st["detail_ms"][:3]],
                                "barrier_ms_block0": round(st["detail_ms"][4], 3),
                                "reference_walk_envelopes_per_run": st["reference_walked"],
                                "own_step_bytes_per_run": st["step_bytes"],
                                "woken_and_nuclei_per_run": st["active_grown"],
                                "entries_processed_per_run": st["grains_processed"],
                                "wake_keys_scanned_per_run": st["keys_scanned"],
                                "liquid_count_decrements_per_run": st["decrements"],
                                "zero_count_events_per_run": st["zero_events"],
                                "list_compactions_per_run": st["compactions"],
                                "parallelism": f"replicas x{args.gpus}", "e2e_field_matches": same}, case),
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "traffic": traffic, "peak_kind": f"{peak_kind} burst copy",
                     "kernel": "plain_persistent_kernel (one launch per run)",
                     "algorithmic_bytes_per_launch": sum(alg_bytes) / len(alg_bytes)},
        "e2e": {"value": e2e_total / e2e_time, "unit": UNIT, "h2d_bytes_per_step": int(np.mean(h2d)),
                "d2h_bytes_per_step": int(np.mean(d2h)), "ms_per_step": 1e3 * e2e_time / args.steps},
        "gpu_launches": launches,
        "clocks": clk,
        "wall_s_timed": wall,
    }
    if args.gpus == 1 and dist.rank == 0 and not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline(args.cpu_sample)
    return line


# ----------------------------------------------------------------------------
# FE-coupled remelting workload (pbf_500)
# ----------------------------------------------------------------------------
PBF_TEXT = ("pbf_500: FE-coupled remelting realm, 500x250x100 cells of 2 um (12.5M) on a columnar baseplate of "
            "2,000 grains (seed 2); one laser pass, Rosenthal frames every 1 us on 10 um FE nodes (P=200 W, A=0.4, "
            "v=1 m/s, k=20, alpha=5e-6, T0=300 K, 1,550 frames generated on the GPU), liquidus 1700 K, solidus "
            "1600 K, bulk sites 1e13 m^-3 (8 K, 2 K), KGT a2=2.03e-4; every CA step to the end of the frames")


def _oracle_pbf_sample(steps: int) -> tuple:
    """The PBF physics on a 250x125x50 block (1/8 of the cells) with a random
    microstructure, the first `steps` CA steps, frames as text."""
    import tempfile

    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import amca_oracle

    cells = (250, 125, 50)
    case = decks.RemeltCase(name="pbf_sample", cells=cells, cell_size=2.0e-6, nucleation=True, seed=2,
                            bulk=(1.0e13, 8.0, 2.0), melting_temperature=1700.0, solidus_temperature=1600.0,
                            a=(0.0, 2.03e-4, 0.0), microstructure="random", termination_time=1.0)
    fr = decks.pbf_frames(cells, case.cell_size, steps + 20)
    wd = tempfile.mkdtemp(prefix="pbf_sample_")
    fr.write(os.path.join(wd, "frames.txt"))
    r = amca_oracle.run_remelt(case, wd, max_steps=steps, fields=False)
    return case.n_interior * r["steps"], r["loop_seconds"], r["steps"]


def cpu_baseline_pbf(steps: int = 40) -> dict:
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import amca_oracle

    amca_oracle.build()
    upd, el, n = _oracle_pbf_sample(steps)
    return {"value": upd / el, "unit": UNIT, "cores": 1, "kind": "port",
            "sample": f"C restatement of the reference, one core: the pbf_500 physics on a 250x125x50 block "
                      f"(random microstructure), its first {n} CA steps, time loop only ({el:.1f} s)"}


def run_reference_arm_pbf(args, dist: Dist):
    if dist.rank != 0:
        return
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import amca_oracle

    amca_oracle.build()
    cores = os.cpu_count() or 1
    ctx = mp.get_context("spawn")
    times, updates = [], []
    with ctx.Pool(cores) as pool:
        for it in range(args.warmup + args.steps):
            res = pool.map(_oracle_pbf_sample, [args.ref_pbf_steps] * cores)
            el = max(r[1] for r in res)
            if it >= args.warmup:
                times.append(el)
                updates.append(sum(r[0] for r in res))
    value = sum(updates) / sum(times)
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * sum(times) / len(times),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": PBF_TEXT, "cells": 12500000},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port",
                         "sample": f"{cores} concurrent single-core runs of the C restatement of the reference, "
                                   f"each the pbf_500 physics on a 250x125x50 block, first {args.ref_pbf_steps} "
                                   f"CA steps, time loop only (the slowest process's loop time)"},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def run_ours_pbf(args, dist: Dist):
    import amca3d_gb300 as A

    dev = dist.local_rank
    case, frames, m = decks.config_pbf_500()
    if args.pbf_block:  # a profiling case with the workload's physics, not the workload
        cells = tuple(int(v) for v in args.pbf_block.split(","))
        case = dataclasses.replace(case, name="pbf_block", cells=cells)
        frames = decks.pbf_frames(cells, case.cell_size, args.pbf_frames or frames.frames)
        m = decks.columnar_microstructure(cells, case.cell_size, case.origin, 2000, 2)
    deck = case.to_yaml()
    rk = frames.rosenthal_kwargs()

    def make():
        r = A.CellularAutomataRealm(deck, seed=case.seed, device=dev)
        r.set_microstructure(m["grain"], m["orient"], m["euler"], m["grain_cell"], m["grain_orient"],
                             expected=m["expected"])
        r.set_rosenthal_frames(**rk)
        return r

    realm = make()
    realm.initialize()
    for _ in range(args.warmup):
        realm.reset()
        realm.run()
    clocks = ClockSampler(dev)
    dist.barrier()
    clocks.start()
    device_ms, updates, ca_steps, alg_bytes, launches = [], [], [], [], 0
    t0 = time.perf_counter()
    for _ in range(args.steps):
        realm.reset()
        realm.run()
        st = realm.stats()
        device_ms.append(st["kernel_ms"])
        updates.append(st["cells"] * st["step"])
        ca_steps.append(st["step"])
        alg_bytes.append(st["algorithmic_bytes"])
        launches += st["launches"] + 1  # step kernel launches + the frame-0 node kernel of the reset
    wall = time.perf_counter() - t0
    dist.barrier()
    clk = clocks.stop()
    st = realm.stats()
    orient = realm.field("orientation_id")
    gstats = grain_stats(orient, case.cells, realm.orientations())
    realm.close()

    pinned = A.PinnedBuffer(case.n_ghost, np.int32)
    e2e_t, e2e_upd, h2d, d2h = [], [], [], []
    for it in range(args.warmup + args.steps):
        t = time.perf_counter()
        r = make()
        r.initialize()
        r.run()
        r.field("orientation_id", out=pinned.array)
        s_ = r.stats()
        r.close()
        el = time.perf_counter() - t
        if it >= args.warmup:
            e2e_t.append(el)
            e2e_upd.append(s_["cells"] * s_["step"])
            h2d.append(s_["h2d_bytes"])
            d2h.append(s_["d2h_bytes"])
    same = bool(np.array_equal(pinned.array, orient))
    pinned.free()

    t_dev = dist.reduce(sum(device_ms) / 1e3, "max")
    upd_total = dist.reduce(float(sum(updates)), "sum")
    e2e_time = dist.reduce(sum(e2e_t), "max")
    e2e_total = dist.reduce(float(sum(e2e_upd)), "sum")
    if dist.rank != 0:
        return
    peak, peak_kind = measured_peak()
    achieved = (sum(alg_bytes) / len(alg_bytes)) / (sum(device_ms) / len(device_ms) / 1e3) / 1e9
    line = {
        "metric": METRIC, "value": upd_total / t_dev, "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": sum(device_ms) / len(device_ms), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": PBF_TEXT if not args.pbf_block else
                   f"pbf_block {args.pbf_block}: the pbf_500 physics on another block (profiling case, not the "
                   f"workload)", "cells": case.n_interior, "seed": case.seed,
                   "l2": "inputs larger than L2: frames 1.6 GB + cell state 1.4 GB per run",
                   "ca_steps_per_run": ca_steps[-1], "grain_objects": st["grains"], **gstats,
                   "nucleations": st["nucleations"], "captures_per_run": st["captures"],
                   "exact_temperatures_per_run": st["generations"], "flagged_per_run": st["active"],
                   "cells_visited_per_run": st["active_grown"], "active_elements_per_run": st["sites_scanned"],
                   "liquid_listed_per_run": st["grains_processed"], "host_velocity_round_trips": st["reserved"],
                   "blocks_per_sm": int(os.environ.get("AMCA_REMELT_BLOCKS_PER_SM", "1")),
                   "phase_ms_update_flags_dt_claim_capture": [round(x, 3) for x in st["phase_ms"][:5]],
                   "host_velocity_wait_ms": round(st["phase_ms"][5], 3),
                   "grid_barrier_ms": round(st["phase_ms"][6], 3),
                   "busy_ms_mean_A_B_C_D_E_host": [round(x, 3) for x in st["detail_ms"][:6]],
                   **({"busy_ms_slowest_A_B_C_D_E_host": [round(x, 3) for x in st["detail_ms"][6:12]],
                       "flag_pass_slowest_ms": round(st["detail_ms"][14], 3)} if PHASE_DETAIL else {}),
                   "block0_newgrain_nucleation_ms": [round(x, 3) for x in st["detail_ms"][12:14]],
                   "parallelism": f"replicas x{args.gpus}", "e2e_field_matches": same},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "traffic": load_traffic("remelt_persistent_pbf_500.json"),
                     "peak_kind": f"{peak_kind} burst copy", "kernel": "remelt_kernel (persistent, one launch per run)",
                     "algorithmic_bytes_per_launch": sum(alg_bytes) / len(alg_bytes)},
        "e2e": {"value": e2e_total / e2e_time, "unit": UNIT, "h2d_bytes_per_step": int(np.mean(h2d)),
                "d2h_bytes_per_step": int(np.mean(d2h)), "ms_per_step": 1e3 * e2e_time / args.steps},
        "gpu_launches": launches,
        "clocks": clk,
        "wall_s_timed": wall,
    }
    if args.gpus == 1 and dist.rank == 0 and not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline_pbf(args.cpu_pbf_steps)
    return line


# ----------------------------------------------------------------------------
# Batched instances (batched_64)
# ----------------------------------------------------------------------------
BATCH_TEXT = ("batched_64: 64 independent plain CA instances, cube edges uniform on 32..128 cells of 2 um "
              "(seed 3; 43.8M cells in all), t_dot log-uniform on [-200, -5] K/s, 50..2,000 bulk Gaussian sites "
              "(3 K, 1 K) each, KGT a1=-0.544e-4 a2=2.03e-4, srand seed 0 per instance; every instance to full "
              "solidification, all in one graph-replayed cooperative launch with an autotuned team size")


def _oracle_instance(case) -> tuple:
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import amca_oracle

    t = time.perf_counter()
    r = amca_oracle.run_plain(case, fields=False)
    return case.n_interior * r["steps"], time.perf_counter() - t


def cpu_baseline_batched(count: int = 8) -> dict:
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import amca_oracle

    amca_oracle.build()
    upd, el = 0, 0.0
    for c in decks.config_batched_64()[:count]:
        u, e = _oracle_instance(c)
        upd += u
        el += e
    return {"value": upd / el, "unit": UNIT, "cores": 1, "kind": "port",
            "sample": f"C restatement of the reference, one core: the first {count} of the 64 instances, each to "
                      f"full solidification, one after another ({el:.1f} s)"}


def run_reference_arm_batched(args, dist: Dist):
    if dist.rank != 0:
        return
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import amca_oracle

    amca_oracle.build()
    cores = os.cpu_count() or 1
    todo = sorted(decks.config_batched_64(), key=lambda c: -c.n_interior)  # longest first
    ctx = mp.get_context("spawn")
    times, updates = [], []
    with ctx.Pool(cores) as pool:
        for it in range(args.warmup + args.steps):
            t = time.perf_counter()
            res = list(pool.imap_unordered(_oracle_instance, todo))
            el = time.perf_counter() - t
            if it >= args.warmup:
                times.append(el)
                updates.append(sum(r[0] for r in res))
    value = sum(updates) / sum(times)
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * sum(times) / len(times),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": BATCH_TEXT, "instances": len(todo), "cells": sum(c.n_interior for c in todo)},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port",
                         "sample": f"the whole workload: the 64 instances as single-core runs of the C "
                                   f"restatement of the reference, {cores} at a time, longest first"},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def _batch_grain_stats(realms, decks_) -> dict:
    grains, cells, aligned = 0, 0, 0.0
    for r, c in zip(realms, decks_):
        g = grain_stats(r.field("orientation_id"), c.cells, r.orientations())
        grains += g["grains"]
        cells += c.n_interior
        aligned += g["texture_100_z_15deg"] * c.n_interior
    return {"grains": grains, "mean_grain_cells": cells / max(grains, 1), "texture_100_z_15deg": aligned / cells}


def run_ours_batched(args, dist: Dist):
    import amca3d_gb300 as A

    from amca3d_gb300 import shard

    dev = dist.local_rank
    all_decks = decks.config_batched_64()
    # N GPUs: the 64 instances partitioned over the ranks (longest first), each rank one batch of its share
    mine = shard.partition(all_decks, dist.world)[dist.rank]
    decks_ = [all_decks[i] for i in mine]
    realms = []
    for c in decks_:
        r = A.CellularAutomataRealm(c.to_yaml(), seed=c.seed, device=dev)
        r.initialize()
        realms.append(r)
    batch = A.Batch(realms)
    # three timings per layout: the mixed layouts are planned from per-realm
    # times, and with two a noisy estimate could leave the search above the
    # best uniform team (one run: 88.6 ms mixed against 73.7-79.4 in others)
    batch.tune(repeats=3)
    layout = batch.layout()
    for _ in range(args.warmup):
        batch.run()
    clocks = ClockSampler(dev)
    dist.barrier()
    clocks.start()
    device_ms, updates, alg_bytes = [], [], []
    t0 = time.perf_counter()
    for _ in range(args.steps):
        device_ms.append(batch.run())
        bs = batch.stats()
        updates.append(bs["cell_updates"])
        alg_bytes.append(sum(r.stats()["algorithmic_bytes"] for r in realms))
    wall = time.perf_counter() - t0
    dist.barrier()
    clk = clocks.stop()
    bs = batch.stats()
    per = [r.stats() for r in realms]
    gstats = _batch_grain_stats(realms, decks_)
    orient_last = [r.field("orientation_id") for r in realms[:4]]
    # every instance's result against its own reference run (digests gathered from all ranks)
    local = {c.name: (shard.field_digest(r.field("orientation_id")), r.stats()["step"]) for c, r in zip(decks_, realms)}
    gathered = {}
    for part in dist.gather(local):
        gathered.update(part)
    golden = json.load(open(os.path.join(ROOT, "tests", "golden", "batched_64_golden.json")))
    match = all(gathered.get(k, ("", -1)) == (v["orient_sha256"], v["steps"]) for k, v in golden.items())
    batch.close()

    # the same 64 instances as 64 sequential plain launches (one persistent
    # launch per instance on the whole GPU), device time
    seq_ms = []
    for it in range(2):
        tot = 0.0
        for r in realms:
            r.reset()
            r.run()
            tot += r.stats()["kernel_ms"]
        seq_ms.append(tot)
    seq_same = all(np.array_equal(realms[i].field("orientation_id"), orient_last[i]) for i in range(4))
    for r in realms:
        r.close()

    # end to end through the public API per step: decks -> 64 realms
    # (host sites + H2D) -> one batch run -> every orientation field into
    # pinned host memory -> close
    pinned = [A.PinnedBuffer(c.n_ghost, np.int32) for c in decks_]
    e2e_t, e2e_upd, h2d, d2h = [], [], [], []
    for it in range(args.warmup + args.steps):
        t = time.perf_counter()
        rs = []
        for c in decks_:
            r = A.CellularAutomataRealm(c.to_yaml(), seed=c.seed, device=dev)
            r.initialize()
            rs.append(r)
        with A.Batch(rs) as b:
            b.set_layout(*layout)
            b.run()
            upd = b.stats()["cell_updates"]
        for r, p in zip(rs, pinned):
            r.field("orientation_id", out=p.array)
        sts = [r.stats() for r in rs]
        for r in rs:
            r.close()
        el = time.perf_counter() - t
        if it >= args.warmup:
            e2e_t.append(el)
            e2e_upd.append(upd)
            h2d.append(sum(s_["h2d_bytes"] for s_ in sts))
            d2h.append(sum(s_["d2h_bytes"] for s_ in sts))
    same = all(np.array_equal(pinned[i].array, orient_last[i]) for i in range(4))
    for p in pinned:
        p.free()

    t_dev = dist.reduce(sum(device_ms) / 1e3, "max")
    upd_total = dist.reduce(float(sum(updates)), "sum")
    e2e_time = dist.reduce(sum(e2e_t), "max")
    e2e_total = dist.reduce(float(sum(e2e_upd)), "sum")
    if dist.rank != 0:
        return
    peak, peak_kind = measured_peak()
    ms = sum(device_ms) / len(device_ms)
    achieved = (sum(alg_bytes) / len(alg_bytes)) / (ms / 1e3) / 1e9
    seq = min(seq_ms)
    steps_all = [p_["step"] for p_ in per]
    line = {
        "metric": METRIC, "value": upd_total / t_dev, "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True,
        "scaling": "strong" if dist.world > 1 else "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": BATCH_TEXT, "instances": len(all_decks), "cells": sum(c.n_interior for c in all_decks),
                   "ca_steps_min_mean_max": [min(steps_all), float(np.mean(steps_all)), max(steps_all)],
                   "cell_updates_per_run": bs["cell_updates"], **gstats,
                   "team_size": bs["team_size"], "teams": bs["teams"], "max_blocks": bs["max_blocks"],
                   "cuda_graph": bool(bs["graph"]), "autotune_ms_by_team": bs["tuned"],
                   "autotune_mixed_ms": bs["mixed_ms"], "layout_classes": bs["classes"],
                   "grid_blocks": bs["grid_blocks"],
                   "sequential_plain_ms": seq, "sequential_plain_cell_updates_per_s": bs["cell_updates"] / (seq / 1e3),
                   "speedup_vs_sequential_plain": seq / ms, "sequential_fields_match": seq_same,
                   "e2e_fields_match": same, "all_instances_match_reference": match,
                   "ranks": dist.world, "instances_rank0": len(decks_),
                   "parallelism": "instances partitioned over ranks, longest first" if dist.world > 1 else "1 GPU",
                   "l2": "inputs larger than L2: 64 orientation fields 183 MB + envelope tables 1.9 GB per run"},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "traffic": load_traffic("ca_batched_64.json"), "peak_kind": f"{peak_kind} burst copy",
                     "kernel": "plain_batched_kernel (one launch per run)",
                     "algorithmic_bytes_per_launch": sum(alg_bytes) / len(alg_bytes)},
        "e2e": {"value": e2e_total / e2e_time, "unit": UNIT, "h2d_bytes_per_step": int(np.mean(h2d)),
                "d2h_bytes_per_step": int(np.mean(d2h)), "ms_per_step": 1e3 * e2e_time / args.steps},
        "gpu_launches": 3 * args.steps,  # per run: reset, batched step kernel, control-block gather
        "clocks": clk,
        "wall_s_timed": wall,
    }
    if args.gpus == 1 and dist.rank == 0 and not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline_batched()
    return line


# ----------------------------------------------------------------------------
# Learned thermal model (thermal_1024): plain FE frames vs model frames
# ----------------------------------------------------------------------------
THERMAL_TEXT = ("thermal_1024: FE-coupled remelting realm, 1024x512x256 cells of 2 um (134M) on a columnar baseplate "
                "of 8,000 grains (seed 4); a 5-track raster (100 um hatch, alternating direction, 200 W, 1 m/s), "
                "frames every 1 us on 10 um FE nodes, produced on the GPU a window at a time: the FE field "
                "(Rosenthal of the current pass, the plain run) or the learned thermal model (Fourier-feature MLP, "
                "4x256 SiLU, bf16 tensor cores, trained on the GPU on 50M FE-field samples, seed 4) with the FE "
                "field where its error estimate exceeds 5 K within 100 K of the 1700 K liquidus; liquidus 1700 K, "
                "solidus 1600 K, bulk sites 1e13 m^-3 (8 K, 2 K), KGT a2=2.03e-4; every CA step to the end of the "
                "frames")
# FLOPs of one training sample (forward GEMMs, weight gradients, input gradients of layers 1-3)
TRAIN_FLOP_PER_SAMPLE = 2 * (2 * (128 * 256 + 3 * 256 * 256)) + 2 * 3 * 256 * 256
INFER_FLOP_PER_QUERY = 2 * (128 * 256 + 3 * 256 * 256 + 2 * 256)


def thermal_accuracy(model, scan, frames, t_liq=1700.0, band=100.0, thresh=5.0) -> dict:
    """Model frames against the FE field's frames at a few frames spread over
    the scan: temperature error (K) over nodes whose FE temperature lies in
    the mushy zone (1600-1700 K), from the network alone and after the
    fallback rule."""
    import amca3d_gb300 as A

    sc = A.Scan.of(**scan)
    errs_net, errs_fb, near, fb, ev = [], [], 0, 0, 0
    for frac in (0.12, 0.31, 0.5, 0.69, 0.88):
        f0 = int(frac * (frames - 2))
        net, fe, c_net = model.frames(sc, f0, 2, t_liq, band, 1e30, with_fe=True)
        out, _, c_fb = model.frames(sc, f0, 2, t_liq, band, thresh)
        mushy = (fe >= 1600.0) & (fe <= 1700.0)
        errs_net.append(np.abs(net[mushy] - fe[mushy]))
        errs_fb.append(np.abs(out[mushy] - fe[mushy]))
        ev += int(c_fb[0])
        near += int(c_fb[1])
        fb += int(c_fb[2])
    en, ef = np.concatenate(errs_net), np.concatenate(errs_fb)

    def summ(e):
        return {"median": float(np.median(e)), "p95": float(np.percentile(e, 95)), "max": float(e.max()),
                "mean": float(e.mean())} if e.size else {}
    return {"mushy_nodes": int(en.size), "network_K": summ(en), "after_fallback_K": summ(ef),
            "nodes_evaluated": ev, "near_liquidus": near, "fallbacks": fb}


def run_ours_thermal(args, dist: Dist):
    import amca3d_gb300 as A
    from amca3d_gb300.grainstats import grain_stats as gs

    dev = dist.local_rank
    if args.thermal_block:
        cells = tuple(int(v) for v in args.thermal_block.split(","))
        case, scan, m = decks.config_thermal_block("thermal_block", cells, tracks=args.thermal_tracks,
                                                   hatch=1.0e-4, grains=max(60, cells[0] * cells[1] // 65))
    else:
        case, scan, m = decks.config_thermal_1024()
    deck = case.to_yaml()
    spec = decks.thermal_spec()
    tr = dict(decks.THERMAL_TRAIN)
    if args.thermal_train_steps:
        tr["steps"] = args.thermal_train_steps
    model = A.ThermalModel(device=dev, **spec)
    t0 = time.perf_counter()
    st_train = model.train(**tr)
    train_wall = time.perf_counter() - t0
    acc = thermal_accuracy(model, scan, scan["frames"])

    def make(kind):
        r = A.CellularAutomataRealm(deck, seed=case.seed, device=dev)
        r.set_microstructure(m["grain"], m["orient"], m["euler"], m["grain_cell"], m["grain_orient"],
                             expected=m["expected"])
        if kind == "fe":
            r.set_scan_frames(**scan)
        else:
            r.set_thermal_frames(model, 1700.0, 100.0, 5.0, **scan)
        r.initialize()
        return r

    res = {}
    clocks = ClockSampler(dev)
    clocks.start()
    for kind in ("fe", "model"):
        r = make(kind)
        for _ in range(args.warmup):
            r.reset()
            r.run()
        wall = []
        for _ in range(args.steps):
            r.reset()
            t = time.perf_counter()
            r.run()
            wall.append(time.perf_counter() - t)
        st = r.stats()
        res[kind] = dict(stats=st, wall=wall, frames=r.frame_stats(),
                         grains=gs(r.field("orientation_id"), r.orientations(), case.cells))
        r.close()
    clk = clocks.stop()
    model.close()
    if dist.rank != 0:
        return
    upd = {k: v["stats"]["cells"] * v["stats"]["step"] for k, v in res.items()}
    rate = {k: upd[k] / (sum(v["wall"]) / len(v["wall"])) for k, v in res.items()}
    g_fe, g_mod = res["fe"]["grains"], res["model"]["grains"]
    line = {
        "metric": METRIC, "value": rate["model"], "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1e3 * sum(res["model"]["wall"]) / len(res["model"]["wall"]),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64 CA, bf16 tensor-core model",
        "data": "synthetic",
        "config": {"workload": THERMAL_TEXT if not args.thermal_block else
                   f"thermal_block {args.thermal_block}, {args.thermal_tracks} tracks: the thermal_1024 physics on "
                   f"another block (profiling case, not the workload)", "cells": case.n_interior,
                   "frames": scan["frames"], "fe_nodes": int(np.prod(scan["nodes"])),
                   "plain_fe_frames_cell_updates_per_s": rate["fe"], "model_frames_cell_updates_per_s": rate["model"],
                   "model_vs_plain": rate["model"] / rate["fe"],
                   "ca_steps": {k: v["stats"]["step"] for k, v in res.items()},
                   "run_ms": {k: 1e3 * sum(v["wall"]) / len(v["wall"]) for k, v in res.items()},
                   "ca_kernel_ms": {k: v["stats"]["kernel_ms"] for k, v in res.items()},
                   "grain_stats_plain": g_fe, "grain_stats_model": g_mod,
                   "grain_stats_rel_diff": {"grains": abs(g_mod["grains"] - g_fe["grains"]) / max(g_fe["grains"], 1),
                                            "mean_size": abs(g_mod["mean_size_cells"] - g_fe["mean_size_cells"])
                                            / max(g_fe["mean_size_cells"], 1e-30),
                                            "frac_100z_abs": abs(g_mod["frac_100z"] - g_fe["frac_100z"])},
                   "model_frames": res["model"]["frames"], "temperature_error": acc,
                   "training": {**st_train, "wall_s": train_wall,
                                "samples_per_s": st_train["samples_seen"] / (st_train["ms"] / 1e3),
                                "tflops": st_train["samples_seen"] * TRAIN_FLOP_PER_SAMPLE / (st_train["ms"] / 1e3)
                                / 1e12, **tr},
                   "model_flop_per_query": INFER_FLOP_PER_QUERY},
        "clocks": clk,
    }
    print(json.dumps(line), flush=True)


def emit(line) -> None:
    if line is not None:
        print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--cpu-sample", type=int, default=128, help="edge of the CPU-baseline sample block")
    ap.add_argument("--ref-sample", type=int, default=96, help="edge of each reference-arm sample block")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-extra", action="store_true",
                    help="uniform_320 only: leave out the pbf_500 and batched_64 results of the default line")
    ap.add_argument("--extra-steps", type=int, default=3, help="timed runs of each extra workload")
    ap.add_argument("--extra-warmup", type=int, default=3, help="warm-up runs of each extra workload (>= 3)")
    ap.add_argument("--workload", choices=["uniform_320", "pbf_500", "batched_64", "thermal_1024"],
                    default="uniform_320")
    ap.add_argument("--thermal-block", default="", help="X,Y,Z cells: run the thermal_1024 physics on another block "
                                                        "(profiling only, not the workload)")
    ap.add_argument("--thermal-tracks", type=int, default=5)
    ap.add_argument("--thermal-train-steps", type=int, default=0, help="override the training steps")
    ap.add_argument("--cpu-pbf-steps", type=int, default=40, help="CA steps of the pbf_500 CPU-baseline sample")
    ap.add_argument("--ref-pbf-steps", type=int, default=20, help="CA steps of each pbf_500 reference-arm sample")
    ap.add_argument("--pbf-block", default="", help="X,Y,Z cells: run the pbf_500 physics on another block "
                                                    "(profiling captures only, not the workload)")
    ap.add_argument("--pbf-frames", type=int, default=0, help="frames of the --pbf-block case")
    ap.add_argument("--cells", type=int, default=320,
                    help="edge of the cubic block to run (320 = the measured workload; smaller blocks keep the "
                         "workload's physics and are for profiling captures only)")
    args = ap.parse_args()
    dist = Dist()
    try:
        if args.workload == "thermal_1024":
            if args.impl == "reference":
                print(json.dumps({"impl": "reference", "unavailable": "the reference has no learned thermal model; "
                                  "its CPU path of this workload's physics is the pbf_500 reference arm"}))
            else:
                run_ours_thermal(args, dist)
        elif args.workload == "pbf_500":
            if args.impl == "reference":
                run_reference_arm_pbf(args, dist)
            else:
                emit(run_ours_pbf(args, dist))
        elif args.workload == "batched_64":
            if args.impl == "reference":
                run_reference_arm_batched(args, dist)
            else:
                emit(run_ours_batched(args, dist))
        elif args.impl == "reference":
            run_reference_arm(args, dist)
        else:
            line = run_ours(args, dist)
            if line is not None and args.gpus == 1 and not args.no_extra and args.cells == 320:
                # the other two workloads of the metric ride along on one GPU, each with its own
                # timing, clocks and roofline (K and W of their own, kept short)
                sub = argparse.Namespace(**vars(args))
                sub.steps, sub.warmup = args.extra_steps, max(3, args.extra_warmup)
                for key, fn in (("pbf_500", run_ours_pbf), ("batched_64", run_ours_batched)):
                    extra = fn(sub, dist)
                    if extra is not None:
                        line[key] = {k: v for k, v in extra.items()
                                     if k not in ("metric", "unit", "n_gpus", "higher_is_better", "scaling",
                                                  "vs_baseline", "data")}
            emit(line)
    finally:
        dist.close()


if __name__ == "__main__":
    main()
