"""Full-size pin of the pbf_500 workload (FE-coupled remelting realm,
500 x 250 x 100 cells on a 2,000-grain columnar baseplate, one Rosenthal
laser pass over 1,550 frames), from the UNMODIFIED reference.

The deck, the frames (the reference's text format) and the baseplate restart
file are those that amca3d_gb300.decks.config_pbf_500() describes and that
bench.py --workload pbf_500 runs through amca_set_rosenthal_frames and
amca_set_microstructure. The reference (oracle/_ref/amca3d_np1_dump, built by
``make -C oracle ref-dump``) runs it at np=1 with seed 2; its state probe
records the realm every EVERY CA steps and at the end of the run
(AMCA_DUMP_EVERY, AMCA_DUMP_FINAL), and this script reduces each record to
SHA-256 digests of the orientation, grain-id and melted fields, the grain
table and the Euler angles, with the step, time, dt and counts.

With --oracle the C restatement (oracle/amca_oracle.c, pinned per step to the
reference on the six small remelting decks) runs the same files instead and
gives the final record; its digests are stored beside the reference's under
"oracle" so the two can be compared.

Output: tests/golden/pbf_500_golden.json. A reference run takes hours on one
core (9.6e10 cell updates).

Usage: python tests/golden/make_pbf_golden.py --workdir DIR [--prepare-only]
                                              [--ref] [--oracle] [--every N]
"""
from __future__ import annotations

import argparse
import hashlib
import json
import os
import subprocess
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))
from amca3d_gb300 import decks  # noqa: E402

REF_BIN = os.path.join(ROOT, "oracle", "_ref", "amca3d_np1_dump")
OUT_JSON = os.path.join(HERE, "pbf_500_golden.json")
GRAIN_REC = np.dtype([("id", "<i4"), ("cell", "<i4"), ("orient", "<i4"), ("active", "u1"),
                      ("xc", "<f8"), ("yc", "<f8"), ("zc", "<f8"), ("length", "<f8")])


def sha(a) -> str:
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def grain_table_digest(g: np.ndarray) -> str:
    """Digest of the grain records without the 'active' flag (the coupled
    path never reads it), in a packed little-endian layout."""
    out = np.zeros(len(g), dtype=[("id", "<i4"), ("cell", "<i4"), ("orient", "<i4"),
                                  ("xc", "<f8"), ("yc", "<f8"), ("zc", "<f8"), ("length", "<f8")])
    for k in out.dtype.names:
        out[k] = g[k]
    return sha(out)


def record_summary(step, t, dt, orient, grain, melted, grains, euler) -> dict:
    return dict(step=int(step), time=float(t).hex(), dt=float(dt).hex(), ngrains=int(len(grains)),
                norient=int(len(euler) // 3), orient=sha(orient.astype("<i4")), grain=sha(grain.astype("<i4")),
                melted=sha(melted.astype("u1")), grains=grain_table_digest(grains), euler=sha(euler.astype("<f8")))


def prepare(workdir: str) -> None:
    """Write Inputfile.i, frames.txt and baseplate0.txt for pbf_500 (skipped
    when a file is already complete: the frames take minutes to write)."""
    os.makedirs(workdir, exist_ok=True)
    case, frames, m = decks.config_pbf_500()
    with open(os.path.join(workdir, "Inputfile.i"), "w") as f:
        f.write(case.to_yaml())
    done = os.path.join(workdir, ".prepared")
    if os.path.exists(done):
        return
    decks.write_restart(os.path.join(workdir, case.microstructure), m, case.origin, case.cells, case.cell_size)
    frames.write(os.path.join(workdir, os.path.basename(case.frames_file)))
    open(done, "w").close()


def iter_records(path: str):
    """Stream the probe's records (oracle/ref_probe/state_dump.cpp layout)."""
    with open(path, "rb") as f:
        def take(n):
            b = f.read(n)
            if len(b) != n:
                raise ValueError("truncated dump")
            return b

        while True:
            magic = f.read(4)
            if not magic:
                return
            if magic == b"AMCT":
                n = int(np.frombuffer(take(4), "<i4")[0])
                f.seek(28 * n, os.SEEK_CUR)
                continue
            if magic != b"AMCD":
                raise ValueError(f"bad record magic {magic!r}")
            step = int(np.frombuffer(take(4), "<i4")[0])
            t, dt, _maxdt = np.frombuffer(take(24), "<f8")
            n, ng, no, nn = (int(v) for v in np.frombuffer(take(16), "<i4"))
            orient = np.frombuffer(take(4 * n), "<i4")
            grain = np.frombuffer(take(4 * n), "<i4")
            f.seek(8 * n + n, os.SEEK_CUR)  # temperature, cooling
            melted = np.frombuffer(take(n), "u1")
            f.seek(n, os.SEEK_CUR)  # liquid-neighbour flags
            grains = np.frombuffer(take(GRAIN_REC.itemsize * ng), GRAIN_REC)
            euler = np.frombuffer(take(24 * no), "<f8")
            f.seek(8 * nn, os.SEEK_CUR)
            yield record_summary(step, t, dt, orient, grain, melted, grains, euler)


def run_reference(workdir: str, every: int) -> dict:
    dump = os.path.join(workdir, "state.bin")
    if os.path.exists(dump):
        os.remove(dump)
    env = dict(os.environ, AMCA_SEED="2", AMCA_DUMP=dump, AMCA_DUMP_EVERY=str(every), AMCA_DUMP_FINAL="1")
    t0 = time.time()
    with open(os.path.join(workdir, "run.log"), "w") as log:
        r = subprocess.run([REF_BIN, "-i", "Inputfile.i", "-o", "ref.log"], cwd=workdir, env=env,
                           stdout=log, stderr=subprocess.STDOUT)
    wall = time.time() - t0
    if r.returncode != 0:
        raise RuntimeError(f"reference failed ({r.returncode}); see {workdir}/run.log")
    recs = list(iter_records(dump))
    final = recs[-1]
    checkpoints = [rc for rc in recs[:-1] if rc["step"] != final["step"]]
    return dict(source="unmodified reference (oracle/_ref/amca3d_np1_dump), np=1, seed 2",
                wall_seconds=round(wall, 1), final=final, checkpoints=checkpoints)


def run_oracle(workdir: str) -> dict:
    import amca_oracle

    amca_oracle.build()
    case, _frames, _m = decks.config_pbf_500()
    t0 = time.time()
    r = amca_oracle.run_remelt(case, workdir, fields=True)
    wall = time.time() - t0
    # the oracle reports fields, counts and the final time; grain table and Euler angles are not exported
    final = dict(step=int(r["steps"]), time=float(r["time"]).hex(), dt=float(r["last_dt"]).hex(),
                 ngrains=int(r["num_grains"]), norient=int(r["num_orient"]),
                 orient=sha(r["orient"].astype("<i4")), grain=sha(r["grain"].astype("<i4")),
                 melted=sha(r["melted"].astype("u1")))
    return dict(source="C restatement (oracle/amca_oracle.c), one core", wall_seconds=round(wall, 1), final=final)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--workdir", required=True)
    ap.add_argument("--prepare-only", action="store_true")
    ap.add_argument("--ref", action="store_true", help="run the unmodified reference")
    ap.add_argument("--oracle", action="store_true", help="run the C restatement")
    ap.add_argument("--every", type=int, default=1000, help="reference checkpoint interval (CA steps)")
    ap.add_argument("--out", default=OUT_JSON, help="JSON file to update")
    args = ap.parse_args()
    prepare(args.workdir)
    if args.prepare_only:
        return
    golden = json.load(open(args.out)) if os.path.exists(args.out) else {}
    case, frames, _m = decks.config_pbf_500()
    golden.update(cells=list(case.cells), seed=case.seed, frames=frames.frames)
    if args.oracle:
        golden["oracle"] = run_oracle(args.workdir)
        print("oracle:", json.dumps(golden["oracle"]["final"]))
    if args.ref:
        golden["reference"] = run_reference(args.workdir, args.every)
        print("reference:", json.dumps(golden["reference"]["final"]))
    with open(args.out, "w") as f:
        json.dump(golden, f, indent=1, sort_keys=True)


if __name__ == "__main__":
    main()
