"""The flush on the GPU against the oracle's restatement: the same meetings
go into both (the GPU's, which the parity tests show equal the oracle's),
both flush at the same steps, and every output must match byte for byte:
packed CTF keys, sids, CTF capacities and metadata, bitmaps, the oversize
buffer's keys, boxes and bitmap."""
import numpy as np
import pytest

from glint_pipeline_gb300 import Configuration, DeviceBench, GlintError
from oracle.bindings import Store
from workloads import case_config, make_points

pytestmark = pytest.mark.gpu

INFO = ("kv_count", "key_bytes", "oversize_kv_count", "oversize_start_time_min", "oversize_start_time_max",
        "oversize_end_time_min", "oversize_end_time_max", "sid_count", "oversize_oid_count", "end_time_min",
        "cur_time", "bits_outside")


def gpu_bench(name, **kw):
    cfgd = case_config(name)
    c = Configuration(num_objects=cfgd["num_objects"], grid_capacity=cfgd["grid_capacity"],
                      grid_amplify=cfgd["grid_amplify"], num_meeting_buckets=cfgd["num_meeting_buckets"],
                      reach_distance=cfgd["reach_distance"], min_meet_time=cfgd["min_meet_time"],
                      schema_update_delay=cfgd["schema_update_delay"], kv_capacity=1 << 22)
    for k, v in kw.items():
        setattr(c, k, v)
    return c


def compare(gs, os_, oinfo, where):
    gi = gs["info"]
    for f in INFO:
        assert getattr(gi, f) == getattr(oinfo, f), f"{where}: info.{f} {getattr(gi, f)} != {getattr(oinfo, f)}"
    for k in ("keys", "sids", "ctf_capacity", "bitmaps", "o_keys", "o_bitmap"):
        assert gs[k].tobytes() == os_[k].tobytes(), f"{where}: {k}"
    assert gs["ctfs"].tobytes() == os_["ctfs"].tobytes(), f"{where}: ctfs"
    assert gs["o_boxes"].view(np.uint32).tobytes() == os_["o_boxes"].view(np.uint32).tobytes(), f"{where}: o_boxes"


def run(name, steps, flush_at=(), auto_restriction=None, dprob=100.0, max_meet=4096):
    box, pts = make_points(name, steps)
    cfgd = case_config(name)
    kw = dict(dProbFalse=dprob, max_meet_time=max_meet)
    if auto_restriction:
        kw.update(auto_flush=True, kv_restriction=auto_restriction)
    g = DeviceBench(gpu_bench(name, **kw), box, pts[0])
    st = Store(cfgd["num_objects"], box, first_end_time_min=cfgd["min_meet_time"], kv_capacity=1 << 22,
               dProbFalse=dprob, max_meet_time=max_meet)
    flushes = 0
    for t in range(steps):
        s = g.step(pts[t], t)
        st.add_meetings(g.meetings())
        if auto_restriction:
            due = st.kv_count > auto_restriction
            assert bool(s.flushed) == due, f"step {t}: flushed {s.flushed}, due {due}"
            if due:
                rc, oi = st.flush(t)
                assert rc == 0
                compare(g.store(), st.result(oi), oi, f"auto flush at {t}")
                flushes += 1
        elif t in flush_at:
            gi = g.flush()
            rc, oi = st.flush(t)
            assert rc == 0
            compare(g.store(), st.result(oi), oi, f"flush at {t}")
            assert gi.kv_count == oi.kv_count
            flushes += 1
    g.close()
    st.close()
    return flushes


def test_flush_matches_oracle():
    assert run("dense_20k", 50, flush_at=(20, 35, 49)) == 3


def test_flush_small_100k():
    assert run("small_100k", 60, flush_at=(30, 59)) == 2


def test_flush_oversize_buffer():
    assert run("dense_20k", 40, flush_at=(25, 39), dprob=2e-9) == 2


def test_auto_flush_matches_oracle():
    assert run("dense_20k", 45, auto_restriction=3_000) >= 2


def test_flush_outside_reference_domain_is_refused():
    box, pts = make_points("dense_20k", 30)
    g = DeviceBench(gpu_bench("dense_20k", max_meet_time=8), box, pts[0])
    for t in range(30):
        g.step(pts[t], t)
    with pytest.raises(GlintError):
        g.flush()
    g.close()


@pytest.mark.parametrize("case", ["dense_20k", "dense_20k_oversize", "small_100k", "collide_20k"])
def test_device_flush_matches_reference_gpu_kernels(case):
    """The device flush against the reference's OWN GPU kernels on the same
    workload (tests/golden/ref_gpu_flush.npz, made by running the
    reference's unmodified geometry.cu flush): every flush's packed keys,
    sids, capacities, CTF records, bitmaps and oversize buffer."""
    import os

    import make_ref_gpu_golden as G
    g = np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "ref_gpu_flush.npz"))
    steps, flush_at, dprob, max_meet, split = G.FLUSH_CASES[case]
    name = G.workload(case)
    box, pts = make_points(name, steps)
    dev = DeviceBench(gpu_bench(name, dProbFalse=dprob, max_meet_time=max_meet, CTF_count=split * split,
                                split_num=split), box, pts[0])
    k = 0
    for t in range(steps):
        dev.step(pts[t], t)
        if t in flush_at:
            dev.flush()
            s = dev.store()
            assert [int(getattr(s["info"], f)) for f in G.INFO] == g[f"{case}/info"][k].tolist(), f"t={t}"
            assert G.flush_digests(s) == g[f"{case}/digests"][k].tolist(), f"t={t}"
            k += 1
    assert k == len(flush_at)
    dev.close()
