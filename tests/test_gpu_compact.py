"""Compaction of kept blocks on the GPU (glint_store_compact; merge_dump,
tools/compaction.cpp:729-1215) against the oracle's restatement in the same
stable tie order (oracle/glint_compact_oracle.c, itself pinned against the
reference's own merge_dump), on blocks the device flushed: every array of
the merged block bit for bit, its files read back, and queries over it."""
import os

import numpy as np
import pytest

from glint_pipeline_gb300 import Configuration, DeviceBench, GlintError, write_store_files
from oracle.bindings import compact_blocks
from workloads import case_config, make_points

pytestmark = pytest.mark.gpu


def build(name, steps, flush_at, dprob=100.0, keep=16):
    box, pts = make_points(name, steps)
    cfgd = case_config(name)
    c = Configuration(num_objects=cfgd["num_objects"], grid_capacity=cfgd["grid_capacity"],
                      grid_amplify=cfgd["grid_amplify"], num_meeting_buckets=cfgd["num_meeting_buckets"],
                      reach_distance=cfgd["reach_distance"], min_meet_time=cfgd["min_meet_time"],
                      schema_update_delay=cfgd["schema_update_delay"], kv_capacity=1 << 22, store_keep=keep,
                      dProbFalse=dprob)
    g = DeviceBench(c, box, pts[0])
    for t in range(steps):
        g.step(pts[t], t)
        if t in flush_at:
            g.flush()
    return g, cfgd["num_objects"], np.asarray(box, np.float64)


def check_equal(got, want):
    np.testing.assert_array_equal(got["sids"], want["sids"])
    for f in want["ctfs"].dtype.names:
        if f != "reserved":
            np.testing.assert_array_equal(got["ctfs"][f], want["ctfs"][f], err_msg=f)
    np.testing.assert_array_equal(got["bitmaps"], want["bitmaps"])
    np.testing.assert_array_equal(got["keys"], want["keys"])
    np.testing.assert_array_equal(got["o_keys"], want["o_keys"])
    np.testing.assert_array_equal(got["o_boxes"].view(np.uint32), want["o_boxes"].view(np.uint32))
    np.testing.assert_array_equal(got["o_bitmap"], want["o_bitmap"])


def compact_and_check(g, n, box, first, count, split_num):
    src = [g.block(i) for i in range(first, first + count)]
    rc, want = compact_blocks(src, n, box, split_num)
    assert rc == 0
    nblocks = g.store_blocks()
    info = g.compact(first, count, split_num)
    assert g.store_blocks() == nblocks - count + 1
    got = g.block(first)
    check_equal(got, want)
    assert got["times"] == [int(v) for v in want["times8"][:4]]
    assert got["o_times"] == [int(v) for v in want["times8"][4:]]
    for k in ("kv_count", "key_bytes", "padding", "x_part", "y_part", "sid_count"):
        assert info[k] == want[k], k
    assert info["oversize_kv_count"] == want["o_count"]
    return got, want, info


@pytest.mark.parametrize("name,steps,flush_at,first,count,split_num,dprob", [
    ("dense_20k", 50, (20, 35, 49), 0, 3, 4, 100.0),
    ("dense_20k", 50, (20, 35, 49), 1, 2, 7, 100.0),
    ("reach_8k", 40, (19, 39), 0, 2, 3, 100.0),       # object 0 has keys: its repeats
    ("dense_20k", 40, (19, 39), 0, 2, 5, 2e-9),        # oversize buffers to merge
    ("collide_20k", 40, (19, 39), 0, 2, 1, 100.0),     # one CTF
])
def test_compaction_matches_oracle(name, steps, flush_at, first, count, split_num, dprob):
    g, n, box = build(name, steps, flush_at, dprob)
    try:
        got, want, info = compact_and_check(g, n, box, first, count, split_num)
        if name == "reach_8k":
            assert info["padding"] > 0 and want["sids"][0] >= 2
        if dprob < 1:
            assert info["oversize_kv_count"] > 0
    finally:
        g.close()


def test_compacting_a_compacted_block():
    """a compacted block is a source like any other: its CTF ends are
    absolute (end_time_min 0) and object 0's repeats are keys of object 0"""
    g, n, box = build("reach_8k", 60, (19, 39, 59))
    try:
        compact_and_check(g, n, box, 0, 2, 3)
        compact_and_check(g, n, box, 0, 2, 4)
        assert g.store_blocks() == 1
    finally:
        g.close()


def test_compacted_block_files_and_queries(tmp_path):
    g, n, box = build("dense_20k", 50, (20, 35, 49))
    try:
        g.compact(0, 3, 5)
        blk = g.block(0)
        raid, meta = str(tmp_path / "r"), str(tmp_path / "m")
        for d in (raid + "0", raid + "1", meta):
            os.makedirs(d)
        g.dump_block(0, raid, meta, "6G", 0)
        # the files hold what the block holds, and the same files written from
        # the host arrays are identical
        h = DeviceBench(g.config, box, make_points("dense_20k", 1)[1][0])
        try:
            h.load_store(raid, meta, "6G", 0, ctf_count=25)
            back = h.block(0)
            check_equal(back, blk)
            assert back["times"] == blk["times"]
            # queries: the device index of the compacted block against the
            # index the loader rebuilds from the files
            rng = np.random.default_rng(9)
            qs = [(rng.choice(n, k, replace=False).astype(np.uint32), hops, 0, 0)
                  for k, hops in [(1, 3), (50, 2), (500, 1), (2000, 3)]]
            qs.append((np.array([0], np.uint32), 2, 0, 0))   # object 0 and its repeats
            a, sa = g.query(qs)
            b, sb = h.query(qs)
            assert sa == sb
            for x, y in zip(a, b):
                for hx, hy in zip(x, y):
                    np.testing.assert_array_equal(hx, hy)
        finally:
            h.close()
        os.makedirs(tmp_path / "w" / "r0")
        os.makedirs(tmp_path / "w" / "r1")
        os.makedirs(tmp_path / "w" / "m")
        write_store_files(blk, blk["info"], n, str(tmp_path / "w" / "r"), str(tmp_path / "w" / "m"), "6G", 0)
        for f in sorted(os.listdir(tmp_path / "m")):
            a = open(tmp_path / "m" / f, "rb").read()
            b = open(tmp_path / "w" / "m" / f, "rb").read()
            if "_CTB" in f:   # the CTB record's times are written only by the block dump
                a, b = a[128:], b[128:]
            assert a == b, f
    finally:
        g.close()


def test_compaction_domain_errors():
    g, n, box = build("reach_8k", 40, (19, 39))
    try:
        with pytest.raises(GlintError):
            g.compact(1, 2, 3)            # past the kept blocks
        with pytest.raises(GlintError, match="too few objects"):
            g.compact(0, 2, 60)
        assert g.store_blocks() == 2      # untouched
        g.compact(0, 2, 2)
        assert g.store_blocks() == 1
    finally:
        g.close()


def test_compaction_past_2_19_objects():
    """with more than 2^19 objects the flush's packed keys can keep sid bits
    above the object id (key_bit rounds up past it); the merge reads the id
    as the reference's readers do, and still equals the oracle bit for bit"""
    from glint_pipeline_gb300.tracegen import SEED_SCALE, TraceGenerator
    n, steps = 600_000, 36
    gen = TraceGenerator(SEED_SCALE + 0x600, n)
    box, pts = gen.box(), gen.steps(steps)
    c = Configuration(num_objects=n, num_meeting_buckets=1 << 26, store_keep=8)
    g = DeviceBench(c, box, pts[0])
    try:
        for t in range(steps):
            g.step(pts[t], t)
            if t % 12 == 11:
                g.flush()
        blocks = [g.block(i) for i in range(g.store_blocks())]
        # some CTF leaves room above its id field, and a key there carries a sid bit
        carried = 0
        for b in blocks:
            off = 0
            for m in b["ctfs"]:
                kb, cnt = int(m["key_bit"]) // 8, int(m["CTF_kv_capacity"])
                top = 2 * int(m["id_bit"]) + int(m["duration_bit"]) + int(m["end_bit"]) + int(m["mbr_bit"])
                if int(m["key_bit"]) > top and cnt:
                    raw = b["keys"][off:off + kb * cnt].reshape(cnt, kb)
                    hi = np.array([int.from_bytes(r.tobytes(), "little") >> top for r in raw[:200]])
                    carried += int((hi != 0).sum())
                off += kb * cnt
        assert carried > 0
        box = np.asarray(box, np.float64)
        compact_and_check(g, n, box, 0, len(blocks), 12)
    finally:
        g.close()


def test_snapshot_keeps_a_compacted_block(tmp_path):
    """a snapshot holds kept blocks of any CTF count with their bitmaps,
    oversize boxes and record times; the resumed context reads them back
    equal and answers queries alike"""
    g, n, box = build("dense_20k", 50, (20, 35, 49), dprob=2e-9)
    h = None
    try:
        g.compact(0, 2, 4)                 # blocks: compacted (16 CTFs), flushed (100)
        path = str(tmp_path / "ctx.snap")
        g.snapshot(path)
        h = DeviceBench.resume(path, g.config)
        assert h.store_blocks() == g.store_blocks() == 2
        for i in range(2):
            a, b = g.block(i), h.block(i)
            check_equal(b, a)
            assert a["times"] == b["times"] and a["o_times"] == b["o_times"]
        rng = np.random.default_rng(5)
        qs = [(rng.choice(n, k, replace=False).astype(np.uint32), hops, 0, 0) for k, hops in [(10, 3), (400, 2)]]
        x, sx = g.query(qs)
        y, sy = h.query(qs)
        assert sx == sy
        for u, v in zip(x, y):
            for hu, hv in zip(u, v):
                np.testing.assert_array_equal(hu, hv)
    finally:
        if h is not None:
            h.close()
        g.close()
