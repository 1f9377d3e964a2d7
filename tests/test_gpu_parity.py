"""CUDA path vs the CPU oracle, step by step, through the C ABI.

Integer and index outputs must be bit-exact: the meetings identified each
step (pair, start, end, in the reference's bucket order), the f32 meeting
boxes, the check / candidate / contact / bucket counts, the schema records,
both free stacks and the whole bucket table.  The golden fixtures (produced
by the reference's own sources) are checked against the GPU directly too.
"""
import os

import numpy as np
import pytest

from glint_pipeline_gb300 import Configuration, DeviceBench, GlintError
from oracle.bindings import Oracle, cantor_inverse, make_config
from workloads import CASES, case_config, digest, make_points

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
EF_INFO = 0x0100  # GLINT_EF_SCHEMA_WINDOW is informational


def gpu_config(cfgd, **kw):
    c = Configuration(num_objects=cfgd["num_objects"], grid_capacity=cfgd["grid_capacity"],
                      grid_amplify=cfgd["grid_amplify"], num_meeting_buckets=cfgd["num_meeting_buckets"],
                      reach_distance=cfgd["reach_distance"], min_meet_time=cfgd["min_meet_time"],
                      schema_update_delay=cfgd["schema_update_delay"])
    for k, v in kw.items():
        setattr(c, k, v)
    return c


def compare_meetings(mo, mg, t):
    a, b = cantor_inverse(mo["key"])
    assert len(mg) == len(mo), f"step {t}: {len(mg)} meetings on GPU, {len(mo)} in the oracle"
    np.testing.assert_array_equal(mg["pid1"], a, err_msg=f"step {t} pid1")
    np.testing.assert_array_equal(mg["pid2"], b, err_msg=f"step {t} pid2")
    np.testing.assert_array_equal(mg["start"], mo["start"], err_msg=f"step {t} start")
    np.testing.assert_array_equal(mg["end"], mo["end"], err_msg=f"step {t} end")
    np.testing.assert_array_equal(mg["mbr"].view(np.uint32), mo["mbr"].view(np.uint32), err_msg=f"step {t} mbr")


def compare_state(o, g):
    c = o.counts()
    sch_o, ss_o, gs_o, gc_o = o.schema()
    sch_g, ss_g, gs_g, gc_g, ssi, gsi = g.schema()
    assert (ssi, gsi) == (c.schema_stack_index, c.grids_stack_index)
    np.testing.assert_array_equal(sch_g["type"], sch_o["type"])
    v = sch_o["type"] != 0
    for f in ("grid_id", "level", "mid_x", "mid_y", "low", "high", "overflow_count", "underflow_count"):
        np.testing.assert_array_equal(sch_g[f][v], sch_o[f][v], err_msg=f)
    br = sch_o["type"] == 1
    np.testing.assert_array_equal(sch_g["children"][br], sch_o["children"][br])
    np.testing.assert_array_equal(ss_g[ssi:], ss_o[ssi:])
    np.testing.assert_array_equal(gs_g[gsi:], gs_o[gsi:])
    np.testing.assert_array_equal(gc_g, gc_o)
    ko, so, eo, mo = o.buckets()
    kg, sg, mg = g.buckets()
    np.testing.assert_array_equal(kg, ko)
    occ = ko != (1 << 62)
    np.testing.assert_array_equal(sg[occ], so[occ])
    np.testing.assert_array_equal(mg[occ].view(np.uint32), mo[occ].view(np.uint32))


def run_parity(name, steps=None, state_every=10, precision_mode=0):
    box, pts = make_points(name, steps)
    cfgd = case_config(name)
    o = Oracle(make_config(**cfgd), box, pts[0])
    g = DeviceBench(gpu_config(cfgd, precision_mode=precision_mode), box, pts[0])
    compare_state(o, g)
    total = 0
    for t in range(pts.shape[0]):
        o.step(pts[t], t)
        st = g.step(pts[t], t)
        c = o.counts()
        assert st.error_flags & ~EF_INFO == 0, f"step {t}: error flags {st.error_flags:#x}"
        assert st.ambiguous == 0
        assert (st.checks, st.candidates, st.contacts) == (c.grid_check_counter, c.candidates, c.contacts), f"step {t}"
        assert (st.num_taken_buckets, st.num_active_meetings) == (c.num_taken_buckets, c.num_active_meetings)
        assert (st.nodes, st.leaves) == (c.schema_stack_index, c.grids_stack_index), f"step {t}"
        compare_meetings(o.meetings(), g.meetings(), t)
        total += st.meetings
        if state_every and (t % state_every == state_every - 1 or t == pts.shape[0] - 1):
            compare_state(o, g)
    g.close()
    o.close()
    return total


@pytest.mark.parametrize("name", ["dense_20k", "collide_20k", "skew_5k", "delay_10k", "reach_8k"])
def test_parity_with_oracle(name):
    assert run_parity(name) > 0


def test_parity_small_100k():
    """The small plain case (100k objects, 100 steps) against the oracle."""
    run_parity("small_100k", state_every=50)


@pytest.mark.parametrize("name", ["dense_20k", "collide_20k", "skew_5k", "reach_8k", "small_100k"])
def test_parity_precision_form(name):
    """FP32 guard-band refine: the same meetings, counts and state as the oracle."""
    run_parity(name, state_every=25, precision_mode=1)


@pytest.mark.parametrize("name,precision_mode", [("dense_20k", 0), ("collide_20k", 1), ("reach_8k", 0)])
def test_active_search_matches_oracle(name, precision_mode):
    """glint_active_search after a step equals the oracle's restatement of the
    reference's multi-search, record for record (bucket order, mbr bits)."""
    box, pts = make_points(name)
    cfgd = case_config(name)
    o = Oracle(make_config(**cfgd), box, pts[0])
    g = DeviceBench(gpu_config(cfgd, precision_mode=precision_mode), box, pts[0])
    rng = np.random.default_rng(11)
    found = 0
    for t in range(pts.shape[0]):
        o.step(pts[t], t)
        g.step(pts[t], t)
        if t % 4 != 3:
            continue
        k = 1 + (t % 3) * 500
        pids = np.concatenate([rng.choice(cfgd["num_objects"], k, replace=False), [1, 1, 2**31]]).astype(np.uint32)
        want = o.active_search(pids)
        got = g.active_search(pids)
        assert got.tobytes() == want.tobytes(), f"step {t}"
        found += len(got)
        if len(want) > 3:
            part = g.active_search(pids, cap=3)
            assert part.tobytes() == want[:3].tobytes()
    assert found > 0
    assert len(g.active_search(np.zeros(0, np.uint32))) == 0
    g.close()
    o.close()


@pytest.mark.parametrize("name", sorted(CASES))
def test_gpu_matches_reference_fixtures(name):
    """The GPU's per-step meetings hash to the reference's (tests/golden)."""
    gold = np.load(os.path.join(GOLDEN, f"{name}.npz"))
    box, pts = make_points(name)
    cfgd = case_config(name)
    g = DeviceBench(gpu_config(cfgd), box, pts[0])
    from glint_pipeline_gb300._abi import MEETING_DTYPE  # noqa: F401
    from oracle.bindings import oracle_lib
    lib = oracle_lib()
    for t in range(pts.shape[0]):
        st = g.step(pts[t], t)
        m = g.meetings()
        keys = np.array([lib.go_cantor(int(a), int(b)) for a, b in zip(m["pid1"], m["pid2"])], dtype=np.uint64)
        assert digest(keys, m["start"], m["end"]) == str(gold["step_digests"][t]), f"{name} step {t}"
        assert (st.checks, st.meetings, st.num_taken_buckets, st.num_active_meetings, st.leaves, st.nodes) == \
            tuple(int(v) for v in gold["counts"][t])
    g.close()


def test_step_device_refuses_host_memory():
    """glint_step_device reads device memory only: a host array is refused
    before anything is enqueued, and the context steps on afterwards as the
    oracle does."""
    box, pts = make_points("dense_20k", 3)
    cfgd = case_config("dense_20k")
    o = Oracle(make_config(**cfgd), box, pts[0])
    g = DeviceBench(gpu_config(cfgd), box, pts[0])
    host = np.ascontiguousarray(pts[0])
    with pytest.raises(GlintError):
        g.step_device(host.ctypes.data, 0)
    for t in range(3):
        o.step(pts[t], t)
        g.step(pts[t], t)
        compare_meetings(o.meetings(), g.meetings(), t)
    g.close()
    o.close()


def test_device_generator_matches_host():
    import ctypes
    from glint_pipeline_gb300 import _abi
    from glint_pipeline_gb300.tracegen import TraceGenerator
    n = 50_000
    host = TraceGenerator(0x5151, n)
    ref = host.steps(25)
    g2 = TraceGenerator(0x5151, n)
    lib = _abi.lib()
    pb = g2.params_bytes()
    ob = g2.objects_bytes()
    h = ctypes.c_void_p()
    assert lib.glint_gen_create(pb, len(pb), ob, n, len(ob) // n, 0, ctypes.byref(h)) == 0
    import glint_pipeline_gb300 as gp
    bench_cfg = gp.Configuration(num_objects=n)
    b = gp.DeviceBench(bench_cfg, host.box(), ref[0])  # owns a stream and device memory we can borrow
    out = np.zeros((n, 2))
    # generate each step on the bench's stream into a device buffer and compare a host copy
    for t in range(25):
        dptr = _device_buffer(n)
        assert lib.glint_gen_step(h, ctypes.c_void_p(dptr.ptr), ctypes.c_void_p(b.stream)) == 0
        dptr.copy_to_host(out, b.stream)
        np.testing.assert_array_equal(out, ref[t], err_msg=f"step {t}")
        dptr.free()
    lib.glint_gen_destroy(h)
    b.close()


class _device_buffer:
    """A raw cudaMalloc'd buffer through libcudart (test helper)."""

    def __init__(self, n):
        import ctypes
        self.rt = _cudart()
        p = ctypes.c_void_p()
        assert self.rt.cudaMalloc(ctypes.byref(p), ctypes.c_size_t(16 * n)) == 0
        self.ptr = p.value
        self.n = n

    def copy_to_host(self, out, stream):
        import ctypes
        assert self.rt.cudaDeviceSynchronize() == 0
        assert self.rt.cudaMemcpy(out.ctypes.data_as(ctypes.c_void_p), ctypes.c_void_p(self.ptr),
                                  ctypes.c_size_t(16 * self.n), 2) == 0

    def free(self):
        import ctypes
        self.rt.cudaFree(ctypes.c_void_p(self.ptr))


def _cudart():
    import ctypes
    import glob
    for cand in ["libcudart.so", "libcudart.so.13"] + glob.glob("/usr/local/cuda/lib64/libcudart.so*"):
        try:
            return ctypes.CDLL(cand)
        except OSError:
            continue
    raise OSError("libcudart not found")


def test_graph_mode_parity():
    """The step captured once as a CUDA graph and replayed from a fixed device
    input buffer gives the oracle's meetings, counts and state."""
    import ctypes
    name = "dense_20k"
    box, pts = make_points(name, 40)
    cfgd = case_config(name)
    o = Oracle(make_config(**cfgd), box, pts[0])
    g = DeviceBench(gpu_config(cfgd, use_graph=True, precision_mode=1), box, pts[0])
    rt = _cudart()
    n = cfgd["num_objects"]
    buf = ctypes.c_void_p()
    assert rt.cudaMalloc(ctypes.byref(buf), ctypes.c_size_t(16 * n)) == 0
    try:
        for t in range(pts.shape[0]):
            o.step(pts[t], t)
            host = np.ascontiguousarray(pts[t])
            assert rt.cudaMemcpy(buf, host.ctypes.data_as(ctypes.c_void_p), ctypes.c_size_t(16 * n), 1) == 0
            g.step_device(buf.value, t)
            st = g.sync()
            c = o.counts()
            assert st.error_flags & ~EF_INFO == 0
            assert (st.checks, st.candidates, st.contacts) == (c.grid_check_counter, c.candidates, c.contacts), t
            compare_meetings(o.meetings(), g.meetings(), t)
        compare_state(o, g)
    finally:
        rt.cudaFree(buf)
        g.close()
        o.close()


def test_precision_probe_screen_agrees_with_fp64():
    """glint_precision_probe: on every sampled pair the FP32 screen's decision
    equals the FP64 test's (or defers to it inside the band), the screen's
    distance error near the reach stays inside the guard band, and the report
    does not depend on the precision mode the steps ran in."""
    name = "dense_20k"
    box, pts = make_points(name, 12)
    cfgd = case_config(name)
    n = cfgd["num_objects"]
    reps = {}
    for mode in (0, 1):
        g = DeviceBench(gpu_config(cfgd, precision_mode=mode), box, pts[0])
        try:
            for t in range(pts.shape[0]):
                g.step(pts[t], t)
            reps[mode] = {s: g.precision_probe(s) for s in (1, 7)}
        finally:
            g.close()
    for s, rep in reps[1].items():
        expect = sum(min(32, n - 1 - i) for i in range(0, n, s))
        assert rep["pairs"] == expect, (s, rep)
        assert rep["mismatches"] == 0, rep
        assert 0 < rep["contacts"] <= rep["pairs"], rep
        assert rep["in_band"] <= rep["pairs"], rep
        assert 0.0 < rep["max_abs_err_near_m"] < rep["max_band_m"] < 1e-4, rep
        assert rep["max_abs_err_near_m"] <= rep["max_abs_err_m"], rep
        assert rep == reps[0][s], (rep, reps[0][s])


def test_meetings_into_pinned_buffer():
    """glint_meetings into page-locked memory from glint_host_alloc gives the
    same records as into a fresh array, step after step (the buffer is
    reused)."""
    from glint_pipeline_gb300 import pinned_empty
    from glint_pipeline_gb300._abi import MEETING_DTYPE
    name = "dense_20k"
    box, pts = make_points(name, 20)
    cfgd = case_config(name)
    g = DeviceBench(gpu_config(cfgd, precision_mode=1), box, pts[0])
    buf = pinned_empty(cfgd["num_objects"], MEETING_DTYPE)
    seen = 0
    try:
        for t in range(pts.shape[0]):
            g.step(pts[t], t)
            a = g.meetings()
            b = g.meetings(out=buf)
            assert b.base is not None and b.shape == a.shape
            np.testing.assert_array_equal(a.view(np.uint8), b.view(np.uint8))
            seen += a.shape[0]
        assert seen > 0
    finally:
        g.close()


def test_pipelined_stepping_matches_plain_steps():
    """glint_pipe_*: with the next step's points copied while the current
    step runs and meetings written into page-locked result buffers, every
    step's meetings and counts, the automatic flushes in between and the
    final store equal those of plain glint_step calls."""
    from glint_pipeline_gb300 import Pipe, pinned_empty
    name = "dense_20k"
    box, pts = make_points(name, 36)
    cfgd = case_config(name)
    n = cfgd["num_objects"]
    kw = dict(precision_mode=1, auto_flush=True, kv_restriction=3000, kv_capacity=1 << 20, store_keep=2)
    a = DeviceBench(gpu_config(cfgd, **kw), box, pts[0])
    b = DeviceBench(gpu_config(cfgd, **kw), box, pts[0])
    host = pinned_empty((pts.shape[0], n, 2), np.float64)
    host[:] = pts
    pipe = Pipe(b, result_capacity=n)
    try:
        pipe.submit(host[0], 0)
        flushes = 0
        for t in range(pts.shape[0]):
            sa = a.step(pts[t], t)
            ma = a.meetings()
            if t + 1 < pts.shape[0]:
                pipe.submit(host[t + 1], t + 1)
            sb, mb = pipe.result(t)
            assert sb.cur_time == t
            assert (sa.contacts, sa.new_keys, sa.meetings, sa.flushed, sa.kv_count) == \
                   (sb.contacts, sb.new_keys, sb.meetings, sb.flushed, sb.kv_count), t
            np.testing.assert_array_equal(ma.view(np.uint8), mb.view(np.uint8), err_msg=f"step {t}")
            flushes += sa.flushed
        assert flushes >= 2
        sa_, sb_ = a.store(), b.store()
        for k in ("keys", "sids", "ctfs", "bitmaps", "o_keys"):
            np.testing.assert_array_equal(sa_[k], sb_[k], err_msg=k)
    finally:
        pipe.close()
        a.close()
        b.close()


def test_trace_files_through_pipe_match_oracle(tmp_path):
    """The reference's trace chunk files, read ahead by glint_trace_* and fed
    to glint_pipe_*, give the oracle's meetings step by step, across a chunk
    boundary."""
    from glint_pipeline_gb300 import Pipe, TraceFiles, write_trace_files
    name = "dense_20k"
    box, pts = make_points(name, 130)
    cfgd = case_config(name)
    n = cfgd["num_objects"]
    prefix = str(tmp_path / "trace_")
    write_trace_files(prefix, 0, pts)
    o = Oracle(make_config(**cfgd), box, pts[0])
    g = DeviceBench(gpu_config(cfgd, precision_mode=1), box, pts[0])
    tr = TraceFiles(prefix, n, 80, 40)
    pipe = Pipe(g)
    try:
        for t in range(80):
            o.step(pts[t], t)
            g.step(pts[t], t)
        pipe.submit(tr.step(80), 80)
        for t in range(80, 120):
            o.step(pts[t], t)
            if t + 1 < 120:
                pipe.submit(tr.step(t + 1), t + 1)
            st, m = pipe.result(t)
            c = o.counts()
            assert (st.candidates, st.contacts) == (c.candidates, c.contacts), t
            compare_meetings(o.meetings(), m, t)
    finally:
        pipe.close()
        tr.close()
        g.close()
        o.close()


def test_snapshot_resume_continues_bit_for_bit(tmp_path):
    """glint_snapshot_save between steps and glint_snapshot_load in a new
    context: the resumed context's next steps give the same meetings, counts,
    flushes, schema, bucket table, store and query answers as the saved
    context's own next steps."""
    name = "dense_20k"
    box, pts = make_points(name, 50)
    cfgd = case_config(name)
    cfg = gpu_config(cfgd, precision_mode=1, auto_flush=True, kv_restriction=3000, kv_capacity=1 << 20,
                     store_keep=3)
    a = DeviceBench(cfg, box, pts[0])
    b = None
    try:
        for t in range(30):
            a.step(pts[t], t)
        path = str(tmp_path / "ctx.snap")
        a.snapshot(path)
        b = DeviceBench.resume(path, cfg)
        np.testing.assert_array_equal(a.meetings().view(np.uint8), b.meetings().view(np.uint8))
        flushes = 0
        for t in range(30, 50):
            sa, sb = a.step(pts[t], t), b.step(pts[t], t)
            assert (sa.candidates, sa.contacts, sa.new_keys, sa.meetings, sa.flushed, sa.kv_count, sa.leaves,
                    sa.nodes) == (sb.candidates, sb.contacts, sb.new_keys, sb.meetings, sb.flushed, sb.kv_count,
                                  sb.leaves, sb.nodes), t
            np.testing.assert_array_equal(a.meetings().view(np.uint8), b.meetings().view(np.uint8), err_msg=str(t))
            flushes += sa.flushed
        assert flushes >= 1
        for x, y in zip(a.schema(), b.schema()):
            np.testing.assert_array_equal(np.asarray(x), np.asarray(y))
        (ka, sa_start, ma), (kb, sb_start, mb) = a.buckets(), b.buckets()
        np.testing.assert_array_equal(ka, kb)
        occupied = ka != (1 << 62)
        np.testing.assert_array_equal(sa_start[occupied], sb_start[occupied])
        np.testing.assert_array_equal(ma[occupied].view(np.uint32), mb[occupied].view(np.uint32))
        sa_, sb_ = a.store(), b.store()
        for k in ("keys", "sids", "ctfs", "bitmaps", "o_keys", "o_boxes", "o_bitmap"):
            np.testing.assert_array_equal(sa_[k], sb_[k], err_msg=k)
        assert a.store_blocks() == b.store_blocks() == 3
        rng = np.random.default_rng(5)
        qs = [(rng.choice(cfgd["num_objects"], 200, replace=False).astype(np.uint32), 2, 0, 0)]
        ra, rb = a.query(qs), b.query(qs)
        for h in range(2):
            np.testing.assert_array_equal(ra[0][0][h], rb[0][0][h])
    finally:
        if b is not None:
            b.close()
        a.close()
