"""Independent instances over GPUs: the one way the CA path shards.

A single domain does not split under bit-exactness (the capture cascade
would need a halo exchange per generation), but independent instances (a
batch of decks, seeds or parameter sweeps) go to GPUs whole: no collective
touches the data path, only the results are gathered on the host.

The partition is longest-processing-time first: instances sorted by
estimated work, each given to the rank with the least work so far. The work
estimate of a uniform-cooling instance is cells x steps, with the step count
modelled as edge^0.84 |t_dot|^-0.3 (a power law fitted to the measured step
counts of the batched_64 family: edges 32-128, t_dot -5..-200 K/s).
"""
from __future__ import annotations

import hashlib
from typing import List, Sequence

import numpy as np


def instance_work(case) -> float:
    nx, ny, nz = case.cells
    edge = (nx * ny * nz) ** (1.0 / 3.0)
    return float(nx * ny * nz) * edge ** 0.84 * abs(case.t_dot) ** -0.3


def partition(cases: Sequence, world: int) -> List[List[int]]:
    """Instance indices per rank; every instance once, ranks' loads balanced."""
    if world < 1:
        raise ValueError("world must be >= 1")
    order = sorted(range(len(cases)), key=lambda i: (-instance_work(cases[i]), i))
    load = [0.0] * world
    parts: List[List[int]] = [[] for _ in range(world)]
    for i in order:
        r = min(range(world), key=lambda k: (load[k], k))
        parts[r].append(i)
        load[r] += instance_work(cases[i])
    return parts


def field_digest(field: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(field, np.int32).tobytes()).hexdigest()
