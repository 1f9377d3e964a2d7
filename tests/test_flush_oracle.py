"""The flush restatement (oracle/glint_flush_oracle.c) against the reference's
own CTF encoding (tracing/step_merge.cpp, compiled into oracle/_ref):
CTF::get_ctf_bits for every file's bit widths and grids, CTF::serial_mbr and
CTF::serial_key for every packed key whose box lies inside its file's box,
and CTF::binary_search / the search_SSTable walk reading the packed files.
The reference produces the store only on its GPU path, which cannot run
here, so the sort/STR/reduction steps are pinned by restatement only."""
import ctypes
import os

import numpy as np
import pytest

from oracle.bindings import Oracle, Store, cantor_inverse, make_config, ref_available
from workloads import case_config, make_points

REC = np.dtype([("pid1", "<u4"), ("pid2", "<u4"), ("start", "<u4"), ("end", "<u4"), ("mbr", "<f4", (4,))])
BITS = ("key_bit", "id_bit", "duration_bit", "end_bit", "low_x_bit", "low_y_bit", "edge_bit", "mbr_bit", "x_grid",
        "y_grid")


def meeting_records(m):
    a, b = cantor_inverse(m["key"])
    r = np.zeros(len(m), REC)
    r["pid1"], r["pid2"], r["start"], r["end"], r["mbr"] = a, b, m["start"], m["end"], m["mbr"]
    return r


def run_store(name="dense_20k", steps=40, flush_at=(24, 39), **store_kw):
    box, pts = make_points(name, steps)
    cfgd = case_config(name)
    o = Oracle(make_config(**cfgd), box, pts[0])
    st = Store(cfgd["num_objects"], box, first_end_time_min=cfgd["min_meet_time"], **store_kw)
    flushes = []
    for t in range(steps):
        o.step(pts[t], t)
        st.add_meetings(meeting_records(o.meetings()))
        if t in flush_at:
            rc, info = st.flush(t)
            res = st.result(info) if rc == 0 else None
            keys, boxes = st.sorted_keys(info) if rc == 0 else (None, None)
            flushes.append((t, rc, info, res, keys, boxes))
    o.close()
    return box, flushes, st


def unpack_keys(raw16):
    lo = raw16[:, :8].copy().view("<u8").ravel()
    hi = raw16[:, 8:].copy().view("<u8").ravel()
    return lo, hi


def test_flush_properties():
    box, flushes, st = run_store()
    for t, rc, info, res, keys, boxes in flushes:
        assert rc == 0, f"flush at {t}: rc {rc}"
        cap = res["ctf_capacity"]
        assert int(cap.sum()) == info.kv_count > 0
        assert (cap > 0).all()
        lo, hi = unpack_keys(keys[: info.kv_count])
        order = np.lexsort((lo, hi))
        assert (order == np.arange(len(order))).all(), "CTF keys not sorted"
        sid = (hi >> np.uint64(52)) & np.uint64(0xfff)
        first = np.concatenate([[0], np.cumsum(cap)[:-1]]).astype(np.int64)
        cap = cap.astype(np.int64)
        for c in range(len(cap)):
            assert (sid[first[c]:first[c] + cap[c]] == c + 2).all()
        assert info.key_bytes == int((cap.astype(np.int64) * res["ctfs"]["key_bit"] // 8).sum())
        assert (res["ctfs"]["end_time_max"] == t).all()
    st.close()


@pytest.mark.skipif(not ref_available(), reason="reference sources not on this machine")
def test_flush_encoding_matches_reference_ctf():
    from oracle.bindings import ref_lib
    lib = ref_lib()
    box, flushes, st = run_store()
    m4 = np.asarray(box, np.float64)
    checked = skipped = 0
    for t, rc, info, res, keys, boxes in flushes:
        assert rc == 0
        cap = res["ctf_capacity"]
        first = np.concatenate([[0], np.cumsum(cap)[:-1]]).astype(np.int64)
        byte0 = np.concatenate([[0], np.cumsum(cap.astype(np.int64) * res["ctfs"]["key_bit"] // 8)[:-1]])
        for c, meta in enumerate(res["ctfs"]):
            mbr = np.ascontiguousarray(meta["ctf_mbr"], np.float32)
            bits = np.zeros(10, np.uint16)
            size = ctypes.c_uint32()
            lib.ref_ctf_bits(mbr.ctypes.data, m4.ctypes.data, st.cfg.num_objects, 4096, bits.ctypes.data,
                             ctypes.byref(size))
            assert [int(meta[f]) for f in BITS] == [int(b) for b in bits], f"CTF {c} bits"
            assert int(meta["ctf_bitmap_size"]) == size.value
            kb = int(meta["key_bit"]) // 8
            packed = res["keys"][byte0[c]: byte0[c] + cap[c] * kb].reshape(-1, kb)
            lo, hi = unpack_keys(keys[first[c]: first[c] + cap[c]])
            for i in range(0, int(cap[c]), max(1, int(cap[c]) // 64)):
                b = np.ascontiguousarray(boxes[first[c] + i], np.float32)
                if not (b[0] >= mbr[0] and b[1] >= mbr[1] and b[2] <= mbr[2] and b[3] <= mbr[3]):
                    skipped += 1
                    continue
                vm = lib.ref_serial_mbr(mbr.ctypes.data, bits.ctypes.data, b.ctypes.data)
                pid = int(hi[i]) >> 26
                target = int(hi[i]) & ((1 << 26) - 1)
                out = np.zeros(16, np.uint8)
                lib.ref_serial_key(mbr.ctypes.data, bits.ctypes.data, pid, target, int(lo[i]) >> 32,
                                   int(lo[i]) & 0xffffffff, vm, out.ctypes.data)
                assert out[:kb].tobytes() == packed[i].tobytes(), f"CTF {c} key {i}"
                checked += 1
            # the reference's reader finds every object's run of keys
            oids = (hi >> np.uint64(26)) & np.uint64((1 << 26) - 1)
            pk = np.ascontiguousarray(packed)
            for oid in np.unique(oids)[:: max(1, len(np.unique(oids)) // 8)]:
                n = ctypes.c_uint32()
                f = lib.ref_ctf_find(mbr.ctypes.data, bits.ctypes.data, pk.ctypes.data, int(cap[c]), int(oid),
                                     ctypes.byref(n))
                idx = np.nonzero(oids == oid)[0]
                assert f == idx[0] and n.value == len(idx)
    assert checked > 1000 and skipped < checked
    st.close()


def test_flush_oversize_and_domain():
    # a tiny area cut sends objects to the oversize buffer
    box, flushes, st = run_store(flush_at=(30,), dProbFalse=2e-9)
    t, rc, info, res, keys, boxes = flushes[0]
    assert rc == 0 and info.oversize_kv_count > 0 and info.oversize_oid_count > 0
    lo, hi = unpack_keys(keys[info.kv_count:])
    assert (np.lexsort((lo, hi)) == np.arange(len(lo))).all()
    assert res["o_bitmap"].any()
    st.close()
    # meetings longer than max_meet_time shift the reference's CTF ranges: refused
    box, flushes, st = run_store(flush_at=(39,), max_meet_time=8)
    assert flushes[0][1] == -4
    st.close()


REF_GPU_GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "ref_gpu_flush.npz")


@pytest.mark.parametrize("case", ["dense_20k", "dense_20k_oversize", "small_100k", "collide_20k"])
def test_flush_oracle_matches_reference_gpu_kernels(case):
    """The flush restatement against the reference's OWN GPU kernels
    (cuda_identify_meetings and process_with_gpu's flush, run from the
    reference's unmodified geometry.cu; tests/golden/make_ref_gpu_golden.py):
    every flush's packed keys, sids, capacities, CTF records, bitmaps and
    oversize buffer, as digests, plus the counts."""
    import make_ref_gpu_golden as G
    from oracle.bindings import Store
    g = np.load(REF_GPU_GOLDEN)
    res = G.run_flush_case(case, Store, run_ref=False)
    assert [r["t"] for r in res] == g[f"{case}/flush_steps"].tolist()
    for k, r in enumerate(res):
        assert G.info_tuple(r["oracle_info"]) == g[f"{case}/info"][k].tolist(), f"t={r['t']}"
        assert G.flush_digests(r["oracle"]) == g[f"{case}/digests"][k].tolist(), f"t={r['t']}"


@pytest.mark.parametrize("case", ["dense_20k", "reach_8k"])
def test_active_search_oracle_matches_reference_gpu_kernel(case):
    """The active multi-search restatement against the reference's own
    cuda_identify_meetings search (cuda/geometry.cu:605-663) run on the GPU,
    record multisets per step as digests."""
    import make_ref_gpu_golden as G
    from oracle.bindings import Oracle, make_config
    from workloads import case_config, make_points
    g = np.load(REF_GPU_GOLDEN)
    steps, _ = G.SEARCH_CASES[case]
    box, pts = make_points(case, steps)
    cfgd = case_config(case)
    o = Oracle(make_config(**cfgd), box, pts[0])
    digs = []
    for t in range(steps):
        o.step(pts[t], t)
        if t >= 8:
            digs.append(G.digest(G.canonical_search(o.active_search(G.search_pids(case, t)))))
    o.close()
    assert digs == g[f"search/{case}/digests"].tolist()
    assert int(g[f"search/{case}/counts"].sum()) > 0
