"""Batching form: many independent regions advanced together on one GPU
(glint_batch_*), and a small autotuner for per-region settings.

Each region is its own context with its own stream.  A timestep of the whole
batch is one captured CUDA graph: every region's stages up to the refine
stage side by side, one refine launch over the work items of every region in
the FP32-screen form, then every region's remaining stages.
"""
from __future__ import annotations

import ctypes
import time

import numpy as np

from . import _abi
from . import Configuration, DeviceBench, GlintError


class Batch:
    def __init__(self, configs: list[Configuration], mbrs, first_points):
        self.lib = _abi.lib()
        n = len(configs)
        self.configs = configs
        cfgs = (_abi.GlintConfig * n)(*[c.to_c() for c in configs])
        boxes = (_abi.GlintBox * n)()
        for r, m in enumerate(mbrs):
            m = np.asarray(m, np.float64).reshape(4)
            boxes[r].low[0], boxes[r].low[1], boxes[r].high[0], boxes[r].high[1] = m
        self._first = [np.ascontiguousarray(p, dtype=np.float64) for p in first_points]
        ptrs = (ctypes.c_void_p * n)(*[p.ctypes.data for p in self._first])
        h = ctypes.c_void_p()
        st = self.lib.glint_batch_create(n, cfgs, boxes, ptrs, ctypes.byref(h))
        if st != 0:
            raise GlintError(st, "glint_batch_create")
        self.h = h
        self.regions = [DeviceBench._view(self.lib.glint_batch_region(h, r), configs[r]) for r in range(n)]

    def __len__(self):
        return len(self.regions)

    def stream(self, r: int) -> int:
        return self.regions[r].stream

    def step(self, d_points: list[int], cur_time: int):
        arr = (ctypes.c_void_p * len(d_points))(*[int(p) for p in d_points])
        st = self.lib.glint_batch_step(self.h, arr, int(cur_time))
        if st != 0:
            raise GlintError(st, "glint_batch_step")

    def sync(self):
        stats = (_abi.GlintStepStats * len(self.regions))()
        st = self.lib.glint_batch_sync(self.h, stats)
        if st != 0:
            raise GlintError(st, "glint_batch_sync")
        return list(stats)

    def close(self):
        if getattr(self, "h", None):
            for r in self.regions:
                r.h = None
            self.lib.glint_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def autotune(make_config, run_trial, capacities=(32, 50, 128, 512, 1024), load_factors=(0.5, 0.7, 0.9),
             chunks=(64, 128, 256, 512)):
    """Pick (leaf capacity, hash load factor, refine tile width) for one
    region by timing short trials: capacity x load factor at the default
    tile width first, then the tile widths at the best pair.
    make_config(capacity, load_factor, chunk) -> Configuration;
    run_trial(config) -> seconds per step.  Returns ((capacity, load_factor,
    chunk, seconds), table)."""
    table = []

    def trial(cap, lf, chunk):
        t0 = time.perf_counter()
        try:
            sec = run_trial(make_config(cap, lf, chunk))
        except GlintError:
            sec = float("inf")
        table.append({"capacity": cap, "load_factor": lf, "refine_chunk": chunk, "sec_per_step": sec,
                      "trial_s": time.perf_counter() - t0})
        return sec

    best = None
    for cap in capacities:
        for lf in load_factors:
            sec = trial(cap, lf, chunks[0])
            if best is None or sec < best[3]:
                best = (cap, lf, chunks[0], sec)
    for chunk in chunks[1:]:
        sec = trial(best[0], best[1], chunk)
        if sec < best[3]:
            best = (best[0], best[1], chunk, sec)
    return best, table
