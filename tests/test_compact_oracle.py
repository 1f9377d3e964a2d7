"""Compaction of stored blocks: the oracle's restatement of the reference's
merge_dump (tools/compaction.cpp:729-1215, oracle/glint_compact_oracle.c)
against merge_dump itself, built from the tool's own source into oracle/_ref
and run on blocks written in the reference's file layout.  The oracle's
exact-tie mode (the C++ library's std::sort with the reference's
comparators) must reproduce the reference's files bit for bit; the stable
mode (the device path's order) is checked for the layout merge_dump gives.
Host code only; no device is needed."""
import os
import subprocess
import sys

import numpy as np
import pytest

from glint_pipeline_gb300 import write_store_files
from oracle.bindings import BIT_BYTES, compact_blocks, ref_available, ref_lib
from test_flush_oracle import run_store

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
_CACHE = {}


def source_blocks(name="dense_20k", steps=60, flush_at=(19, 39, 59), **kw):
    """flushed blocks of one oracle run, as compaction sources"""
    key = (name, steps, flush_at, tuple(sorted(kw.items())))
    if key not in _CACHE:
        box, flushes, st = run_store(name=name, steps=steps, flush_at=flush_at, **kw)
        st.close()
        blocks = []
        for t, rc, info, res, keys, boxes in flushes:
            assert rc == 0, (name, t, rc)
            b = dict(res)
            b["o_times"] = [info.oversize_start_time_min, info.oversize_start_time_max,
                            info.oversize_end_time_min, info.oversize_end_time_max]
            b["times"] = [0, 0, 0, 0]   # straight_dump leaves the CTB's own times zero
            blocks.append((info, b))
        _CACHE[key] = (np.asarray(box, np.float64), blocks)
    box, blocks = _CACHE[key]
    return box, [(i, dict(b)) for i, b in blocks]


def ctf_fields(res, c):
    """(oid, target, duration, end) of every key of CTF c"""
    m = res["ctfs"][c]
    kb = int(m["key_bit"]) // 8
    start = int(np.sum(res["ctfs"]["CTF_kv_capacity"][:c].astype(np.int64) *
                       (res["ctfs"]["key_bit"][:c].astype(np.int64) // 8)))
    raw = res["keys"][start:start + kb * int(m["CTF_kv_capacity"])].reshape(-1, kb)
    out = []
    mb, eb, db, ib = (int(m[f]) for f in ("mbr_bit", "end_bit", "duration_bit", "id_bit"))
    for r in raw:
        k = int.from_bytes(r.tobytes(), "little") >> mb
        end = k & ((1 << eb) - 1)
        k >>= eb
        dur = k & ((1 << db) - 1)
        k >>= db
        tgt = k & ((1 << ib) - 1)
        out.append((k >> ib, tgt, dur, end))
    return np.array(out, np.int64).reshape(-1, 4)


def source_key_counts(blocks, n):
    """CTF keys per object over the sources"""
    cnt = np.zeros(n, np.int64)
    for _, b in blocks:
        for c in range(len(b["ctfs"])):
            f = ctf_fields(b, c)
            if len(f):
                cnt += np.bincount(f[:, 0], minlength=n)
    return cnt


@pytest.mark.parametrize("split_num", [1, 2, 5])
def test_compacted_layout(split_num):
    box, blocks = source_blocks(name="reach_8k", steps=40, flush_at=(19, 39))
    n = blocks[0][1]["sids"].shape[0]
    rc, res = compact_blocks([b for _, b in blocks], n, box, split_num)
    assert rc == 0
    C = split_num * split_num
    cap = res["ctfs"]["CTF_kv_capacity"].astype(np.int64)
    assert int(cap.sum()) == res["kv_count"]
    assert res["key_bytes"] == int((cap * (res["ctfs"]["key_bit"].astype(np.int64) // 8)).sum())
    src = source_key_counts(blocks, n)
    sids = res["sids"].astype(np.int64)
    have = src > 0
    # objects with CTF keys are placed (all but the last of the STR order)
    assert int((sids >= 2).sum()) == int(have.sum()) == res["sid_count"] + 1
    assert ((sids >= 2) == have).all()
    assert src[0] > 0, "this workload gives object 0 keys, so its repeats are exercised"
    placed = np.zeros(n, np.int64)
    for c in range(C):
        f = ctf_fields(res, c)
        oids = f[:, 0]
        assert (np.diff(oids) >= 0).all(), "a CTF's keys are in object order"
        per = np.bincount(oids, minlength=n)
        placed += per
        for o in np.nonzero(per)[0][1:50]:
            if o == 0:
                continue
            assert sids[o] == c + 2
            assert per[o] == src[o]
            tg = f[oids == o, 1]
            assert (np.diff(tg) >= 0).all(), "an object's keys are in target order"
        if per[0]:
            assert per[0] % src[0] == 0, "object 0's keys repeat whole"
    # every placed object's keys once, object 0's once per unfilled entry
    # more; the last object of the STR order keeps sid 2 and loses its keys
    last = [o for o in np.nonzero(have)[0] if placed[o] == 0]
    assert len(last) <= 1
    extra0 = int(placed[0] - (src[0] if sids[0] >= 2 and 0 not in last else 0))
    assert extra0 == res["padding"] * src[0]
    assert res["kv_count"] == int(src.sum()) - sum(int(src[o]) for o in last) + extra0


def test_bits_above_the_id_are_not_the_id():
    """the flush writes its (sid, oid) field whole above the target, so a
    packed key keeps sid bits above the id where key_bit rounds up past it
    (N > 2^19); they are read as the reference's readers read the id
    (CTF::ctf_get_key_oid), and the merge does not change"""
    box, blocks = source_blocks(name="reach_8k", steps=40, flush_at=(19, 39))
    n = blocks[0][1]["sids"].shape[0]
    bs = [b for _, b in blocks]
    rc, want = compact_blocks(bs, n, box, 3)
    assert rc == 0
    marked = []
    for b in bs:
        b = dict(b)
        keys = b["keys"].copy()
        off = 0
        for m in b["ctfs"]:
            kb, cnt = int(m["key_bit"]) // 8, int(m["CTF_kv_capacity"])
            top = 2 * int(m["id_bit"]) + int(m["duration_bit"]) + int(m["end_bit"]) + int(m["mbr_bit"])
            if int(m["key_bit"]) > top and cnt:
                raw = keys[off:off + kb * cnt].reshape(cnt, kb)
                for r in raw:
                    v = int.from_bytes(r.tobytes(), "little") | (1 << top)   # a sid bit above the id
                    r[:] = np.frombuffer(v.to_bytes(kb, "little"), np.uint8)
            off += kb * cnt
        assert not np.array_equal(keys, b["keys"])
        b["keys"] = keys
        marked.append(b)
    rc2, got = compact_blocks(marked, n, box, 3)
    assert rc2 == 0
    for k in ("sids", "keys", "bitmaps", "o_keys"):
        np.testing.assert_array_equal(got[k], want[k])


def test_domain_errors():
    box, blocks = source_blocks(name="reach_8k", steps=40, flush_at=(19, 39))
    n = blocks[0][1]["sids"].shape[0]
    bs = [b for _, b in blocks]
    assert compact_blocks(bs, n, box, 0)[0] == -2
    assert compact_blocks(bs, n, box, 40)[0] == -2, "a partition size underflows"
    empty = dict(bs[0])
    empty["ctfs"] = empty["ctfs"].copy()
    empty["ctfs"]["CTF_kv_capacity"] = 0
    empty["keys"] = np.zeros(0, np.uint8)
    assert compact_blocks([empty], n, box, 2)[0] == -1


def run_reference(cwd, count, n, CTF_count, box, split_num):
    """merge_dump over <cwd>/m/src_CTB0..count-1 in a child process: the
    tool's per-object sorts open OpenMP teams of 128 threads, which the
    child limits to one (its results do not depend on the thread count)"""
    code = ("import sys, numpy as np\n"
            f"sys.path.insert(0, {REPO!r})\n"
            "from oracle.bindings import ref_lib\n"
            f"box = np.array({[float(v) for v in box]!r}, np.float64)\n"
            f"sys.exit(ref_lib().ref_compact(b'm/src', b'r', b'src', {count}, {n}, {CTF_count}, box.ctypes.data, "
            f"4096, {split_num}, b'm/'))\n")
    env = dict(os.environ, OMP_THREAD_LIMIT="1")
    subprocess.run([sys.executable, "-c", code], cwd=cwd, env=env, check=True, stdout=subprocess.DEVNULL,
                   stderr=subprocess.DEVNULL)


def read_reference(count, n, C, res):
    lib = ref_lib()
    pre = f"{2 * count}G".encode()
    h = lib.ref_store_load(b"m/" + pre, b"r", pre, 0, n, C)
    try:
        out = {"sids": np.zeros(n, np.uint16), "ot": np.zeros(5, np.uint32),
               "o_keys": np.zeros((res["o_count"] + 1, 16), np.uint8),
               "o_boxes": np.zeros((res["o_count"] + 1, 4), np.float32), "o_bitmap": np.zeros(BIT_BYTES, np.uint8),
               "ctfs": np.zeros(C, res["ctfs"].dtype), "bitmaps": np.zeros(C * BIT_BYTES, np.uint8),
               "keys": np.zeros(2 * res["key_bytes"] + (1 << 20), np.uint8)}
        lib.ref_store_get(h, *[out[k].ctypes.data for k in
                               ("sids", "ot", "o_keys", "o_boxes", "o_bitmap", "ctfs", "bitmaps", "keys")])
        return out
    finally:
        lib.ref_store_free(h)


CASES = {
    "dense": dict(name="dense_20k", steps=60, flush_at=(19, 39, 59)),
    "object0": dict(name="reach_8k", steps=40, flush_at=(19, 39)),
    "oversize": dict(name="dense_20k", steps=40, flush_at=(19, 39), dProbFalse=2e-9),
}


@pytest.mark.skipif(not ref_available(), reason="reference sources not on this machine")
@pytest.mark.parametrize("case,split_num,extra", [("dense", 2, False), ("dense", 7, False), ("object0", 3, False),
                                                   ("oversize", 4, False), ("oversize", 3, True)])
def test_oracle_matches_reference_merge_dump(case, split_num, extra, tmp_path, monkeypatch):
    box, blocks = source_blocks(**CASES[case])
    n = blocks[0][1]["sids"].shape[0]
    if extra:
        # an object the second block marks oversize while its keys sit in a
        # CTF: merge_dump sends those keys to its extra oversize list
        b = blocks[1][1]
        b["sids"] = b["sids"].copy()
        cand = np.nonzero(b["sids"] >= 2)[0]
        b["sids"][cand[:3]] = 1
    for d in ("r0", "r1", "m"):
        os.makedirs(tmp_path / d)
    for i, (info, b) in enumerate(blocks):
        write_store_files(b, info, n, str(tmp_path / "r"), str(tmp_path / "m"), "src", i)
    rc, res = compact_blocks([b for _, b in blocks], n, box, split_num, std_ties=True)
    assert rc == 0
    if case == "oversize":
        assert res["o_count"] > 0
    if case == "object0":
        assert res["padding"] > 0
    run_reference(str(tmp_path), len(blocks), n, 100, box, split_num)
    monkeypatch.chdir(tmp_path)   # the reference's paths are short and relative
    C = split_num * split_num
    ref = read_reference(len(blocks), n, C, res)
    np.testing.assert_array_equal(ref["sids"], res["sids"])
    on = res["o_count"]
    assert list(ref["ot"]) == [on] + [int(v) for v in res["times8"][4:]]
    np.testing.assert_array_equal(ref["o_keys"][:on], res["o_keys"])
    np.testing.assert_array_equal(ref["o_boxes"][:on].view(np.uint32), res["o_boxes"].view(np.uint32))
    np.testing.assert_array_equal(ref["o_bitmap"], res["o_bitmap"])
    for f in res["ctfs"].dtype.names:
        if f != "reserved":
            np.testing.assert_array_equal(ref["ctfs"][f], res["ctfs"][f], err_msg=f)
    for c in range(C):
        size = int(res["ctfs"]["ctf_bitmap_size"][c])
        np.testing.assert_array_equal(ref["bitmaps"][c * BIT_BYTES:c * BIT_BYTES + size],
                                      res["bitmaps"][c * BIT_BYTES:c * BIT_BYTES + size])
    np.testing.assert_array_equal(ref["keys"][:res["key_bytes"]], res["keys"])


def test_oracle_matches_golden_compaction():
    """the reference's merge_dump output recorded by
    tests/golden/make_compaction_golden.py (for machines without it)"""
    from workloads import digest
    g = np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "compaction.npz"))
    for case, s in [("object0", 3), ("oversize", 4), ("dense", 5)]:
        box, blocks = source_blocks(**CASES[case])
        n = blocks[0][1]["sids"].shape[0]
        rc, res = compact_blocks([b for _, b in blocks], n, box, s, std_ties=True)
        assert rc == 0
        p = f"{case}_{s}_"
        np.testing.assert_array_equal(res["sids"], g[p + "sids"])
        np.testing.assert_array_equal(res["ctfs"].view(np.uint8).ravel(), g[p + "ctfs"])
        on = res["o_count"]
        assert [on] + [int(v) for v in res["times8"][4:]] == list(g[p + "ot"])
        assert digest(res["keys"]) == str(g[p + "keys_digest"])
        C = s * s
        bits = np.concatenate([res["bitmaps"][c * BIT_BYTES:c * BIT_BYTES + int(res["ctfs"]["ctf_bitmap_size"][c])]
                               for c in range(C)])
        assert digest(bits) == str(g[p + "bitmaps_digest"])
        assert digest(res["o_keys"], res["o_boxes"].view(np.uint32), res["o_bitmap"]) == str(g[p + "o_digest"])
