"""Batching form: regions of different sizes and settings advanced together
(one captured graph per timestep, one refine launch over the work items of
every region in the FP32-screen form) give, region by region, the oracle's
meetings, counts and state, whatever the refine tile width."""
import ctypes

import numpy as np
import pytest

from glint_pipeline_gb300.batch import Batch
from oracle.bindings import Oracle, make_config
from test_gpu_parity import EF_INFO, _cudart, compare_meetings, compare_state, gpu_config
from workloads import case_config, make_points

pytestmark = pytest.mark.gpu

REGIONS = ["dense_20k", "skew_5k", "delay_10k", "reach_8k", "collide_20k"]
# the first region has the largest leaf buffer: the contexts created after it
# must not shrink the refine kernels' shared-memory limit below its need
OVERRIDES = [{"grid_capacity": 300}, {}, {}, {}, {}]


def _run_batch(regions, overrides, modes, chunks, steps, swap_at=None):
    data = [make_points(n, steps) for n in regions]
    cfgs = [dict(case_config(n), **ov) for n, ov in zip(regions, overrides)]
    oracles = [Oracle(make_config(**c), box, pts[0]) for c, (box, pts) in zip(cfgs, data)]
    gcfgs = [gpu_config(c, precision_mode=m, refine_chunk=k) for c, m, k in zip(cfgs, modes, chunks)]
    batch = Batch(gcfgs, [box for box, _ in data], [pts[0] for _, pts in data])
    rt = _cudart()
    bufs = []
    for c in cfgs:
        for _ in range(2):
            b = ctypes.c_void_p()
            assert rt.cudaMalloc(ctypes.byref(b), ctypes.c_size_t(16 * c["num_objects"])) == 0
            bufs.append(b)
    try:
        for t in range(steps):
            # from swap_at on, every other region reads its second buffer:
            # the batch captures its graph again
            use = [bufs[2 * r + (1 if swap_at is not None and t >= swap_at and r % 2 == 0 else 0)]
                   for r in range(len(regions))]
            for r, (box, pts) in enumerate(data):
                host = np.ascontiguousarray(pts[t])
                assert rt.cudaMemcpy(use[r], host.ctypes.data_as(ctypes.c_void_p), ctypes.c_size_t(host.nbytes),
                                     1) == 0
                oracles[r].step(pts[t], t)
            batch.step([b.value for b in use], t)
            stats = batch.sync()
            for r, o in enumerate(oracles):
                st, c = stats[r], o.counts()
                assert st.error_flags & ~EF_INFO == 0, (regions[r], t)
                assert (st.checks, st.candidates, st.contacts) == (c.grid_check_counter, c.candidates, c.contacts), \
                    (regions[r], t)
                compare_meetings(o.meetings(), batch.regions[r].meetings(), t)
        for r, o in enumerate(oracles):
            compare_state(o, batch.regions[r])
    finally:
        for b in bufs:
            rt.cudaFree(b)
        batch.close()
        for o in oracles:
            o.close()


def test_batch_matches_oracle_per_region():
    """Both precision forms side by side, tile widths 16 to 512."""
    _run_batch(REGIONS, OVERRIDES, [r % 2 for r in range(len(REGIONS))], [0, 16, 512, 128, 32], steps=30)


def test_batch_all_screened_one_refine_launch():
    """Every region in the FP32-screen form: one refine launch serves all of
    them; leaf capacities differ (the launch sizes shared memory for the
    largest); the graph is captured again when input buffers change."""
    regions = REGIONS + ["dense_20k", "skew_5k"]
    overrides = OVERRIDES + [{"grid_capacity": 1024}, {"grid_capacity": 32}]
    _run_batch(regions, overrides, [1] * len(regions), [64, 256, 16, 64, 1024, 8, 64], steps=24, swap_at=12)
