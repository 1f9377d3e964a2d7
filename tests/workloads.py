"""Seeded workloads shared by the parity tests and the golden-fixture script."""
from __future__ import annotations

import hashlib

import numpy as np

from glint_pipeline_gb300.tracegen import SEED_SMALL, TraceGenerator

# name -> (seed, objects, steps, generator kind, box extent m, bucket count (0 = 2N), extra config)
CASES = {
    # the small plain case: 100k objects, 100 steps, reach 2 m, min 5, B = 2N
    "small_100k": (SEED_SMALL, 100_000, 100, 0, None, 0, {}),
    # dense 4x4 km box: many splits/merges and cross-leaf checks
    "dense_20k": (0x1234, 20_000, 60, 0, 4000.0, 0, {}),
    # prime bucket count at high load: long probe runs and collisions
    "collide_20k": (0x1235, 20_000, 60, 0, 4000.0, 30011, {}),
    # extreme skew, tiny table: leaf overflow drops and deep probe chains
    "skew_5k": (0x99, 5_000, 80, 1, 2000.0, 7919, {}),
    # delayed schema updates with a small leaf capacity
    "delay_10k": (0x777, 10_000, 50, 0, 3000.0, 0, {"grid_capacity": 20, "schema_update_delay": 2}),
    # larger reach and shorter minimum meeting
    "reach_8k": (0x4242, 8_000, 40, 0, 3000.0, 0, {"reach_distance": 6.0, "min_meet_time": 2}),
}


def make_points(name: str, steps: int | None = None):
    seed, n, t, kind, ext, B, extra = CASES[name]
    g = TraceGenerator(seed, n, kind, extent_m=ext) if ext else TraceGenerator(seed, n, kind)
    return g.box(), g.steps(steps if steps is not None else t)


def case_config(name: str):
    seed, n, t, kind, ext, B, extra = CASES[name]
    cfg = dict(num_objects=n, num_meeting_buckets=B or 2 * n, grid_capacity=50, schema_update_delay=1,
               min_meet_time=5, reach_distance=2.0, grid_amplify=2.0)
    cfg.update(extra)
    return cfg


def digest(*arrays) -> str:
    h = hashlib.sha256()
    for a in arrays:
        a = np.ascontiguousarray(a)
        h.update(str(a.dtype).encode())
        h.update(str(a.shape).encode())
        h.update(a.tobytes())
    return h.hexdigest()
