"""Generates tests/golden/*.npz from the reference's own CPU stages.

Runs the unmodified reference sources (tracing/{filter,refinement,meeting,
workbench}.cpp, built by oracle/build_ref.sh into oracle/_ref) on the seeded
workloads of tests/workloads.py and records, per step, what
workbench::update_meetings identified (key, start, end in emission order),
the check/bucket counts, and digests of the schema and bucket table.  Only
this script reads the reference; the committed fixtures travel to machines
without it.

    python tests/golden/make_golden.py [case ...]
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.dirname(HERE))

from oracle.bindings import Reference, build_ref, make_config  # noqa: E402
from workloads import CASES, case_config, digest, make_points  # noqa: E402

# cases whose full meeting lists are stored; the rest keep per-step digests
FULL = {"dense_20k", "collide_20k", "skew_5k", "delay_10k", "reach_8k"}


def run_case(name: str):
    box, pts = make_points(name)
    cfg = make_config(**case_config(name))
    ref = Reference(cfg, box, pts[0])
    steps = pts.shape[0]
    keys, starts, ends, bounds = [], [], [], [0]
    counts = np.zeros((steps, 6), dtype=np.uint64)
    step_digests = []
    for t in range(steps):
        ref.step(pts[t], t)
        m = ref.meetings()
        c = ref.counts()
        counts[t] = (c.grid_check_counter, c.kv_count, c.num_taken_buckets, c.num_active_meetings,
                     c.grids_stack_index, c.schema_stack_index)
        step_digests.append(digest(m["key"], m["start"], m["end"]))
        if name in FULL:
            keys.append(m["key"])
            starts.append(m["start"])
            ends.append(m["end"])
            bounds.append(bounds[-1] + len(m))
    sch, ss, gs, gc = ref.schema()
    valid = sch["type"] != 0
    bk, bs, be = ref.buckets()
    occ = bk != (1 << 62)
    out = dict(
        counts=counts,
        step_digests=np.array(step_digests),
        points_digest=np.array(digest(pts[0], pts[-1])),
        schema_digest=np.array(digest(sch["type"], sch["grid_id"][valid], sch["level"][valid], sch["mid_x"][valid],
                                      sch["mid_y"][valid], sch["low"][valid], sch["high"][valid])),
        stacks_digest=np.array(digest(ss[counts[-1, 5]:], gs[counts[-1, 4]:])),
        buckets_digest=np.array(digest(bk, bs[occ])),
        x_buffer=np.array(ref.counts().x_buffer),
    )
    if name in FULL:
        out.update(keys=np.concatenate(keys), starts=np.concatenate(starts), ends=np.concatenate(ends),
                   bounds=np.array(bounds, dtype=np.int64))
    ref.close()
    np.savez_compressed(os.path.join(HERE, f"{name}.npz"), **out)
    total = int(counts[:, 1].sum())
    print(f"{name}: {steps} steps, {total} meetings")


def main(argv):
    if build_ref() is None:
        raise SystemExit("the reference sources are not present on this machine")
    names = argv or list(CASES)
    for n in names:
        run_case(n)


if __name__ == "__main__":
    main(sys.argv[1:])
