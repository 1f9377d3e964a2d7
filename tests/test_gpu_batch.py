"""Batching form: regions of different sizes and settings advanced together
(per-region streams and captured step graphs) give, region by region, the
oracle's meetings, counts and state."""
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


def test_batch_matches_oracle_per_region():
    steps = 30
    data = [make_points(n, steps) for n in REGIONS]
    cfgs = [dict(case_config(n), **ov) for n, ov in zip(REGIONS, OVERRIDES)]
    oracles = [Oracle(make_config(**c), box, pts[0]) for c, (box, pts) in zip(cfgs, data)]
    gcfgs = [gpu_config(c, precision_mode=r % 2) for r, c in enumerate(cfgs)]
    batch = Batch(gcfgs, [box for box, _ in data], [pts[0] for _, pts in data])
    rt = _cudart()
    bufs = []
    for c in cfgs:
        b = ctypes.c_void_p()
        assert rt.cudaMalloc(ctypes.byref(b), ctypes.c_size_t(16 * c["num_objects"])) == 0
        bufs.append(b)
    try:
        for t in range(steps):
            for r, (box, pts) in enumerate(data):
                host = np.ascontiguousarray(pts[t])
                assert rt.cudaMemcpy(bufs[r], host.ctypes.data_as(ctypes.c_void_p), ctypes.c_size_t(host.nbytes),
                                     1) == 0
                oracles[r].step(pts[t], t)
            batch.step([b.value for b in bufs], t)
            stats = batch.sync()
            for r, o in enumerate(oracles):
                st, c = stats[r], o.counts()
                assert st.error_flags & ~EF_INFO == 0, (REGIONS[r], t)
                assert (st.checks, st.candidates, st.contacts) == (c.grid_check_counter, c.candidates, c.contacts), \
                    (REGIONS[r], t)
                compare_meetings(o.meetings(), batch.regions[r].meetings(), t)
        for r, o in enumerate(oracles):
            compare_state(o, batch.regions[r])
    finally:
        for b in bufs:
            rt.cudaFree(b)
        batch.close()
        for o in oracles:
            o.close()
