"""Generate the golden fixtures by running the UNMODIFIED AMCA3D reference.

Needs oracle/_ref/amca3d_np1 (make -C oracle ref REF=<checkout>), i.e. the
reference sources compiled against the single-rank shims. For every case in
cases.py it writes the deck, runs the reference at np=1 with AMCA_SEED set
(seed mapping: srand(procID*10000 + seed)), and keeps:
  * <name>.npz: ghost-inclusive cellOrientationID_ / cellGrainID_ /
    cellNucleationDT_ parsed from grainInfo0.txt, plus the step count;
  * plain_golden.json: per case, step count, final grain count and SHA-256
    digests of the int32 orientation / grain fields;
  * outputs_tiny/: every output file of the tiny output deck, verbatim.

With --batched it instead runs the 64 instances of the batched workload
(decks.config_batched_64), one reference process per host core, and writes
batched_64_golden.json: per instance, step count, final grain count and the
SHA-256 digests of its orientation / grain fields.

Usage: python tests/golden/make_golden.py [--large] [--only NAME] [--batched]
"""
from __future__ import annotations

import argparse
import dataclasses
import hashlib
import json
import os
import re
import shutil
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, HERE)
import cases  # noqa: E402

REF_BIN = os.path.join(ROOT, "oracle", "_ref", "amca3d_np1")


def sha(a: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(a, dtype="<i4").tobytes()).hexdigest()


def parse_grain_info(path: str):
    with open(path) as f:
        f.readline()
        head = f.readline().split()
        ncells = int(head[0])
        f.readline()
        grain = np.empty(ncells, np.int32)
        orient = np.empty(ncells, np.int32)
        dtc = np.empty(ncells, np.float64)
        for i in range(ncells):
            t = f.readline().split()
            grain[i] = int(t[1])
            orient[i] = int(t[2])
            dtc[i] = float(t[4])
    return orient, grain, dtc, head


def run_reference(case, workdir: str):
    c = dataclasses.replace(case, microstructure_file="grainInfo.txt")
    deck = os.path.join(workdir, "Inputfile.i")
    with open(deck, "w") as f:
        f.write(c.to_yaml())
    env = dict(os.environ, AMCA_SEED=str(case.seed))
    r = subprocess.run([REF_BIN, "-i", "Inputfile.i", "-o", "run.log"], cwd=workdir, env=env,
                       capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"reference failed on {case.name}: {r.stdout[-2000:]} {r.stderr[-2000:]}")
    log = open(os.path.join(workdir, "run.log")).read()
    steps = [int(m) for m in re.findall(r"Time Step Count: (\d+)", log)]
    grains = re.findall(r"Final Number of Grains:\s*\n\s*(\d+)", log)
    orient, grain, dtc, _ = parse_grain_info(os.path.join(workdir, "grainInfo0.txt"))
    return dict(steps=steps[-1] if steps else 0, final_grains=int(grains[-1]) if grains else 0,
                orient=orient, grain=grain, dtc=dtc)


def _batched_entry(case) -> tuple:
    with tempfile.TemporaryDirectory() as wd:
        res = run_reference(case, wd)
    return case.name, dict(steps=res["steps"], final_grains=res["final_grains"], orient_sha256=sha(res["orient"]),
                           grain_sha256=sha(res["grain"]), cells=list(case.cells), t_dot=case.t_dot,
                           bulk_density=case.bulk[0])


def make_batched() -> None:
    import multiprocessing as mp

    from amca3d_gb300 import decks

    todo = sorted(decks.config_batched_64(), key=lambda c: -c.n_interior)  # longest first
    with mp.get_context("spawn").Pool(os.cpu_count() or 1) as pool:
        out = dict(pool.imap_unordered(_batched_entry, todo))
    with open(os.path.join(HERE, "batched_64_golden.json"), "w") as f:
        json.dump(out, f, indent=1, sort_keys=True)
    print(f"batched_64_golden.json: {len(out)} instances")


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--batched", action="store_true", help="only the 64 instances of the batched workload")
    ap.add_argument("--large", action="store_true", help="also run the 320^3 case (tens of minutes)")
    ap.add_argument("--only", default=None)
    ap.add_argument("--from-dir", nargs=2, metavar=("CASE", "DIR"),
                    help="record a finished reference run of CASE (its directory holds run.log and grainInfo0.txt)")
    args = ap.parse_args()
    if args.batched:
        if not os.path.exists(REF_BIN):
            sys.exit(f"{REF_BIN} missing: run `make -C oracle ref REF=<reference checkout>` first")
        make_batched()
        return
    jpath = os.path.join(HERE, "plain_golden.json")
    golden = json.load(open(jpath)) if os.path.exists(jpath) else {}
    if args.from_dir:
        name, wd = args.from_dir
        case = [c for c in cases.small_cases() + cases.large_cases() if c.name == name][0]
        log = open(os.path.join(wd, "run.log")).read()
        steps = [int(m) for m in re.findall(r"Time Step Count: (\d+)", log)]
        grains = re.findall(r"Final Number of Grains:\s*\n\s*(\d+)", log)
        orient, grain, dtc, _ = parse_grain_info(os.path.join(wd, "grainInfo0.txt"))
        golden[name] = dict(steps=steps[-1], final_grains=int(grains[-1]), orient_sha256=sha(orient),
                            grain_sha256=sha(grain), seed=case.seed, cells=list(case.cells))
        with open(jpath, "w") as f:
            json.dump(golden, f, indent=1, sort_keys=True)
        print(name, golden[name])
        return
    if not os.path.exists(REF_BIN):
        sys.exit(f"{REF_BIN} missing: run `make -C oracle ref REF=<reference checkout>` first")
    todo = cases.small_cases() + (cases.large_cases() if args.large else [])
    for case in todo:
        if args.only and case.name != args.only:
            continue
        with tempfile.TemporaryDirectory() as wd:
            res = run_reference(case, wd)
        entry = dict(steps=res["steps"], final_grains=res["final_grains"], orient_sha256=sha(res["orient"]),
                     grain_sha256=sha(res["grain"]), seed=case.seed, cells=list(case.cells))
        golden[case.name] = entry
        if case.n_ghost <= 300000:
            # the envelope-index field of the larger decks is kept only as a digest
            extra = dict(grain=res["grain"]) if case.n_ghost <= 60000 else {}
            np.savez_compressed(os.path.join(HERE, f"{case.name}.npz"), orient=res["orient"],
                                site_dtc=res["dtc"].astype(np.float32), steps=res["steps"], **extra)
        print(case.name, entry, flush=True)
    # the tiny output deck: keep every file
    oc = cases.output_case()
    if not args.only or args.only == oc.name:
        out_dir = os.path.join(HERE, "outputs_tiny")
        shutil.rmtree(out_dir, ignore_errors=True)
        with tempfile.TemporaryDirectory() as wd:
            deck = os.path.join(wd, "Inputfile.i")
            with open(deck, "w") as f:
                f.write(oc.to_yaml())
            env = dict(os.environ, AMCA_SEED=str(oc.seed))
            subprocess.run([REF_BIN, "-i", "Inputfile.i", "-o", "run.log"], cwd=wd, env=env, check=True,
                           capture_output=True)
            os.makedirs(out_dir)
            for dirpath, _, files in os.walk(wd):
                for fn in files:
                    if fn in ("Inputfile.i", "run.log", "timeLog.dat"):
                        continue
                    src = os.path.join(dirpath, fn)
                    rel = os.path.relpath(src, wd)
                    dst = os.path.join(out_dir, rel)
                    os.makedirs(os.path.dirname(dst), exist_ok=True)
                    shutil.copy(src, dst)
        print("outputs_tiny written")
    with open(jpath, "w") as f:
        json.dump(golden, f, indent=1, sort_keys=True)


if __name__ == "__main__":
    main()
