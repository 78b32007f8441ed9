"""Golden fixtures for the FE-coupled remelting path, from the UNMODIFIED
reference.

Needs oracle/_ref/amca3d_np1_dump (``make -C oracle ref-dump``): the
reference objects linked with a probe on VtrManager::execute that appends
the realm's state after every CA step to $AMCA_DUMP (oracle/ref_probe/
state_dump.cpp). For every fixture in remelt_cases.py this writes the frames,
the deck (and restart file), runs the reference at np=1 with AMCA_SEED set,
and keeps:
  * remelt_golden.json: per case the step count, final grain / orientation
    counts and SHA-256 digests of the voxel element tags and parametric
    coordinates;
  * remelt_<name>.npz: per step the time, dt and maxTimestep, grain and
    orientation counts and 64-bit digests (first 8 bytes of SHA-256) of the
    fields in STEP_FIELDS; the final orientation / grain / melted / cooling /
    liquid-neighbour fields in full.

Usage: python tests/golden/make_remelt_golden.py [--only NAME] [--keep DIR]
"""
from __future__ import annotations

import argparse
import hashlib
import json
import os
import shutil
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, HERE)
import remelt_cases  # noqa: E402

REF_BIN = os.path.join(ROOT, "oracle", "_ref", "amca3d_np1_dump")
GRAIN_DT = np.dtype([("id", "<i4"), ("cell", "<i4"), ("orient", "<i4"), ("active", "u1"),
                     ("xc", "<f8"), ("yc", "<f8"), ("zc", "<f8"), ("length", "<f8")])


STEP_FIELDS = ("orient", "grain", "T", "cooling", "melted", "flag", "grains", "euler")


def sha(a) -> str:
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def d64(a) -> np.uint64:
    """First 8 bytes of the SHA-256 of an array's bytes, as a little-endian integer."""
    return np.frombuffer(hashlib.sha256(np.ascontiguousarray(a).tobytes()).digest()[:8], "<u8")[0]


def read_dump(path: str):
    """Parse the probe's records: (tags, parcoords, [step dicts])."""
    buf = open(path, "rb").read()
    off = 0
    tags = pc = None
    steps = []

    def take(n):
        nonlocal off
        b = buf[off:off + n]
        if len(b) != n:
            raise ValueError("truncated dump")
        off += n
        return b

    while off < len(buf):
        magic = take(4)
        if magic == b"AMCT":
            n = int(np.frombuffer(take(4), "<i4")[0])
            tags = np.frombuffer(take(4 * n), "<i4").copy()
            pc = np.frombuffer(take(24 * n), "<f8").copy()
            continue
        if magic != b"AMCD":
            raise ValueError(f"bad record magic {magic!r} at {off - 4}")
        step = int(np.frombuffer(take(4), "<i4")[0])
        time, dt, maxdt = np.frombuffer(take(24), "<f8")
        n, ng, no, nn = (int(v) for v in np.frombuffer(take(16), "<i4"))
        d = dict(step=step, time=float(time), dt=float(dt), maxdt=float(maxdt), ngrains=ng, norient=no)
        d["orient"] = np.frombuffer(take(4 * n), "<i4").copy()
        d["grain"] = np.frombuffer(take(4 * n), "<i4").copy()
        d["T"] = np.frombuffer(take(8 * n), "<f8").copy()
        d["cooling"] = np.frombuffer(take(n), "u1").copy()
        d["melted"] = np.frombuffer(take(n), "u1").copy()
        d["flag"] = np.frombuffer(take(n), "u1").copy()
        d["grains"] = np.frombuffer(take(GRAIN_DT.itemsize * ng), GRAIN_DT).copy()
        d["euler"] = np.frombuffer(take(24 * no), "<f8").copy()
        d["theta"] = np.frombuffer(take(8 * nn), "<f8").copy()
        if steps and steps[-1]["step"] == step:
            continue  # finalize() writes the last step's output once more
        steps.append(d)
    return tags, pc, steps


def grain_table(g: np.ndarray) -> np.ndarray:
    """Grain records without the 'active' flag (the coupled path never reads it)."""
    out = np.zeros(len(g), dtype=[("id", "<i4"), ("cell", "<i4"), ("orient", "<i4"),
                                  ("xc", "<f8"), ("yc", "<f8"), ("zc", "<f8"), ("length", "<f8")])
    for k in out.dtype.names:
        out[k] = g[k]
    return out


def step_digests(d) -> np.ndarray:
    """64-bit digests of one step's fields, in STEP_FIELDS order."""
    vals = dict(d)
    vals["grains"] = grain_table(d["grains"])
    return np.array([d64(vals[k]) for k in STEP_FIELDS], dtype=np.uint64)


def prepare(fx, workdir: str) -> None:
    fx.frames.write(os.path.join(workdir, os.path.basename(fx.case.frames_file)))
    if fx.columnar_grains:
        remelt_cases.columnar_microstructure(fx.case, fx.columnar_grains, fx.columnar_seed,
                                             os.path.join(workdir, fx.case.microstructure), fx.grainless_mod)
    with open(os.path.join(workdir, "Inputfile.i"), "w") as f:
        f.write(fx.case.to_yaml())


def run_reference(fx, workdir: str):
    prepare(fx, workdir)
    dump = os.path.join(workdir, "state.bin")
    env = dict(os.environ, AMCA_SEED=str(fx.case.seed), AMCA_DUMP=dump)
    r = subprocess.run([REF_BIN, "-i", "Inputfile.i", "-o", "run.log"], cwd=workdir, env=env,
                       capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"reference failed on {fx.case.name}: {r.stdout[-2000:]} {r.stderr[-2000:]}")
    return read_dump(dump)


def output_digests(workdir: str) -> dict:
    """SHA-256 of every output file under workdir (inputs and the log excluded)."""
    skip = {"Inputfile.i", "frames.txt", "run.log", "state.bin", "timeLog.dat"}
    out = {}
    for root, _, files in os.walk(workdir):
        for f in files:
            rel = os.path.relpath(os.path.join(root, f), workdir)
            if rel in skip or rel.startswith("grainInfoIn"):
                continue
            out[rel] = hashlib.sha256(open(os.path.join(root, f), "rb").read()).hexdigest()
    return out


def make_outputs_golden() -> None:
    fx = remelt_cases.output_fixture()
    wd = tempfile.mkdtemp(prefix="remelt_out_")
    try:
        tags, pc, steps = run_reference(fx, wd)
        dig = output_digests(wd)
        with open(os.path.join(HERE, "remelt_outputs.json"), "w") as f:
            json.dump({"steps": len(steps), "files": dig}, f, indent=1, sort_keys=True)
        print(f"remelt_outputs: {len(steps)} steps, {len(dig)} output files")
    finally:
        shutil.rmtree(wd, ignore_errors=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--only", default=None)
    ap.add_argument("--outputs", action="store_true", help="only the output-file digests of output_fixture()")
    ap.add_argument("--keep", default=None, help="keep the run directories under this folder")
    args = ap.parse_args()
    if args.outputs:
        make_outputs_golden()
        return
    out_json = os.path.join(HERE, "remelt_golden.json")
    golden = json.load(open(out_json)) if os.path.exists(out_json) else {}
    for fx in remelt_cases.fixtures():
        if args.only and fx.case.name != args.only:
            continue
        wd = tempfile.mkdtemp(prefix="remelt_")
        try:
            tags, pc, steps = run_reference(fx, wd)
            last = steps[-1]
            golden[fx.case.name] = dict(
                seed=fx.case.seed, cells=list(fx.case.cells), steps=len(steps),
                tags=sha(tags), parcoords=sha(pc),
                final=dict(ngrains=last["ngrains"], norient=last["norient"], time=float(last["time"]).hex()))
            np.savez_compressed(
                os.path.join(HERE, f"{fx.case.name}.npz"), orient=last["orient"], grain=last["grain"],
                melted=last["melted"], cooling=last["cooling"], flag=last["flag"],
                time=np.array([d["time"] for d in steps]), dt=np.array([d["dt"] for d in steps]),
                maxdt=np.array([d["maxdt"] for d in steps]),
                ngrains=np.array([d["ngrains"] for d in steps], np.int32),
                norient=np.array([d["norient"] for d in steps], np.int32),
                digests=np.stack([step_digests(d) for d in steps]), fields=np.array(STEP_FIELDS))
            liquid = int(np.sum(last["orient"] == -1))
            print(f"{fx.case.name}: {len(steps)} steps, {last['ngrains']} grains, {last['norient']} orientations, "
                  f"{liquid} cells at -1, t={last['time']:.3e}")
        finally:
            if args.keep:
                dst = os.path.join(args.keep, fx.case.name)
                shutil.rmtree(dst, ignore_errors=True)
                shutil.copytree(wd, dst)
            shutil.rmtree(wd, ignore_errors=True)
    with open(out_json, "w") as f:
        json.dump(golden, f, indent=1, sort_keys=True)


if __name__ == "__main__":
    main()
