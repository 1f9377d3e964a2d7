"""The reference's OWN GPU kernels against the oracle and the device path.

oracle/build_ref.sh compiles the reference's cuda/geometry.cu, unmodified,
into an sm_103a cubin; oracle/ref_gpu_driver.cpp runs its
cuda_identify_meetings (key generation and the active multi-search) and the
flush of process_with_gpu (set_oid ... write_key_and_mbr) on the GPU.  The
same meetings go through the oracle's restatement (oracle/glint_flush_oracle.c)
and, for the flush, through the device path; every stored byte must agree:
packed CTF keys, sids, CTF capacities and metadata, bitmaps, and the
oversize buffer's keys, boxes and bitmap.  The active multi-search appends
with an atomic counter, so its records are compared as a multiset.

Skipped where the cubin was not built (machines without the reference's
sources and without a copy of oracle/_ref); tests/golden/ref_gpu_flush.npz
carries the same results as digests for those.
"""
import numpy as np
import pytest

from oracle.bindings import Oracle, RefGpu, Store, make_config, ref_gpu_available
from workloads import case_config, make_points

import make_ref_gpu_golden as G

pytestmark = [pytest.mark.gpu,
              pytest.mark.skipif(not ref_gpu_available(), reason="the reference's cubin is not built here")]


@pytest.mark.parametrize("case", sorted(G.FLUSH_CASES))
def test_reference_gpu_flush_equals_oracle(case):
    res = G.run_flush_case(case, Store)
    assert res
    for r in res:
        ref, ora, oi = r["ref"], r["oracle"], r["oracle_info"]
        assert ref["info"].bits_in_slack == 0
        for f in G.INFO:
            assert getattr(ref["info"], f) == getattr(oi, f), f"{case} t={r['t']}: {f}"
        for f in G.FIELDS:
            assert ref[f].tobytes() == ora[f].tobytes(), f"{case} t={r['t']}: {f}"


@pytest.mark.parametrize("case", sorted(G.SEARCH_CASES))
def test_reference_gpu_active_search_equals_oracle(case):
    from glint_pipeline_gb300 import Configuration, DeviceBench
    steps, _ = G.SEARCH_CASES[case]
    box, pts = make_points(case, steps)
    cfgd = case_config(case)
    o = Oracle(make_config(**cfgd), box, pts[0])
    g = DeviceBench(Configuration(num_objects=cfgd["num_objects"], grid_capacity=cfgd["grid_capacity"],
                                  grid_amplify=cfgd["grid_amplify"], num_meeting_buckets=cfgd["num_meeting_buckets"],
                                  reach_distance=cfgd["reach_distance"], min_meet_time=cfgd["min_meet_time"],
                                  schema_update_delay=cfgd["schema_update_delay"]), box, pts[0])
    total = 0
    for t in range(steps):
        o.step(pts[t], t)
        g.step(pts[t], t)
        if t < 8:
            continue
        k, s, e, m = o.buckets()
        occ = k != (1 << 62)
        table = np.zeros(int(occ.sum()), np.dtype([("key", "<u8"), ("start", "<u4"), ("end", "<u4"),
                                                   ("mbr", "<f4", (4,))]))
        table["key"], table["start"], table["end"], table["mbr"] = k[occ], s[occ], e[occ], m[occ]
        pids = G.search_pids(case, t)
        rg = RefGpu(cfgd["num_objects"], box, min_meet_time=cfgd["min_meet_time"])
        ref = G.canonical_search(rg.identify(table, t, cfgd["min_meet_time"], pids))
        rg.close()
        want = G.canonical_search(o.active_search(pids))
        dev = G.canonical_search(g.active_search(pids))
        assert ref.tobytes() == want.tobytes(), f"step {t}"
        assert dev.tobytes() == want.tobytes(), f"step {t}"
        total += len(ref)
    assert total > 0
    o.close()
    g.close()
