"""The store on disk: glint_store_write lays a flushed block out as the
reference's straight_dump does (tracing/process.cpp:254-348), and the
reference's own readers (workbench::load_CTB_meta / load_CTF_meta /
load_CTF_keys, tracing/workbench.cpp:302-325, 639-695, compiled into
oracle/_ref) read it back field for field.  The block is the flush oracle's
restatement of the reference's flush, so no device is needed."""
import os

import numpy as np
import pytest

from glint_pipeline_gb300 import GlintError, write_store_files
from oracle.bindings import ref_available, ref_lib
from test_flush_oracle import run_store

BIT_BYTES = 256 * 256 // 8


def short_dirs(tmp_path, monkeypatch):
    # the reference keeps raid_path in a 24-byte field: paths relative to a
    # scratch working directory
    monkeypatch.chdir(tmp_path)
    raid, meta = "r", "m"
    for d in (raid + "0", raid + "1", meta):
        os.makedirs(d)
    return tmp_path, raid, meta


def block(flush_index=0, **kw):
    box, flushes, st = run_store(**kw)
    st.close()
    t, rc, info, res, keys, boxes = flushes[flush_index]
    assert rc == 0
    return info, res


def test_written_files_have_the_reference_layout(tmp_path, monkeypatch):
    info, res = block()
    root, raid, meta = short_dirs(tmp_path, monkeypatch)
    n = res["sids"].shape[0]
    write_store_files(res, info, n, raid, meta, "6oversize_3600", 0)
    C = res["ctfs"].shape[0]
    kb = res["ctfs"]["key_bit"].astype(np.int64) // 8
    cap = res["ctfs"]["CTF_kv_capacity"].astype(np.int64)
    for i in range(C):
        p = f"{raid}{i % 2}/6oversize_3600_SSTable_0-{i}"
        assert os.path.getsize(p) == kb[i] * cap[i]
        assert os.path.getsize(f"{meta}/6oversize_3600_STcL0-{i}") == 80 + int(res["ctfs"]["ctf_bitmap_size"][i])
    on = int(info.oversize_kv_count)
    assert os.path.getsize(f"{meta}/6oversize_3600_CTB0") == 128 + 2 * n + 16 * on + 16 * on + BIT_BYTES
    # the SSTables concatenated are the packed key buffer
    cat = b"".join(open(f"{raid}{i % 2}/6oversize_3600_SSTable_0-{i}", "rb").read() for i in range(C))
    assert cat == res["keys"].tobytes()


def test_write_refuses_missing_directory():
    info, res = block()
    with pytest.raises(GlintError, match="cannot create"):
        write_store_files(res, info, res["sids"].shape[0], "/nonexistent/r", "/nonexistent/m", "p", 0)


@pytest.mark.skipif(not ref_available(), reason="reference sources not on this machine")
# the default block, and one whose tiny area cut fills the oversize buffer
@pytest.mark.parametrize("case", [{}, {"flush_at": (30,), "dProbFalse": 2e-9}])
def test_reference_loader_reads_written_block(case, tmp_path, monkeypatch):
    info, res = block(**case)
    if "dProbFalse" in case:
        assert info.oversize_kv_count > 0
    root, raid, meta = short_dirs(tmp_path, monkeypatch)
    n = res["sids"].shape[0]
    C = res["ctfs"].shape[0]
    write_store_files(res, info, n, raid, meta, "6oversize_3600", 3)
    lib = ref_lib()
    h = lib.ref_store_load(f"{meta}/6oversize_3600".encode(), raid.encode(), b"6oversize_3600", 3, n, C)
    try:
        on = int(info.oversize_kv_count)
        sids = np.zeros(n, np.uint16)
        ot = np.zeros(5, np.uint32)
        okeys = np.zeros((max(on, 1), 16), np.uint8)
        oboxes = np.zeros((max(on, 1), 4), np.float32)
        obm = np.zeros(BIT_BYTES, np.uint8)
        metas = np.zeros(C, res["ctfs"].dtype)
        bms = np.zeros(C * BIT_BYTES, np.uint8)
        keys = np.zeros(max(res["keys"].size, 1), np.uint8)
        lib.ref_store_get(h, sids.ctypes.data, ot.ctypes.data, okeys.ctypes.data, oboxes.ctypes.data, obm.ctypes.data,
                          metas.ctypes.data, bms.ctypes.data, keys.ctypes.data)
        np.testing.assert_array_equal(sids, res["sids"])
        assert list(ot) == [on, info.oversize_start_time_min, info.oversize_start_time_max,
                            info.oversize_end_time_min, info.oversize_end_time_max]
        np.testing.assert_array_equal(okeys[:on], res["o_keys"][:on])
        np.testing.assert_array_equal(oboxes[:on].view(np.uint32), res["o_boxes"][:on].view(np.uint32))
        np.testing.assert_array_equal(obm, res["o_bitmap"])
        for f in res["ctfs"].dtype.names:
            if f != "reserved":
                np.testing.assert_array_equal(metas[f], res["ctfs"][f], err_msg=f)
        for i in range(C):
            size = int(res["ctfs"]["ctf_bitmap_size"][i])
            np.testing.assert_array_equal(bms[i * BIT_BYTES:i * BIT_BYTES + size],
                                          res["bitmaps"][i * BIT_BYTES:i * BIT_BYTES + size])
        np.testing.assert_array_equal(keys[:res["keys"].size], res["keys"])
        # every object's keys, found by the reference's own search routing
        lo = res["o_keys"][:on, 8:].copy().view("<u8").ravel() if on else np.zeros(0, np.uint64)
        o_pid = ((lo >> np.uint64(26)) & np.uint64((1 << 26) - 1)).astype(np.int64)
        o_count = np.bincount(o_pid, minlength=n) if on else np.zeros(n, np.int64)
        per_ctf = {}
        for i in range(C):
            m = res["ctfs"][i]
            kbytes = int(m["key_bit"]) // 8
            start = int(np.sum(res["ctfs"]["CTF_kv_capacity"][:i].astype(np.int64) *
                               (res["ctfs"]["key_bit"][:i].astype(np.int64) // 8)))
            raw = res["keys"][start:start + kbytes * int(m["CTF_kv_capacity"])].reshape(-1, kbytes)
            shift = int(m["id_bit"] + m["duration_bit"] + m["end_bit"] + m["mbr_bit"])
            vals = [int.from_bytes(r.tobytes(), "little") >> shift & ((1 << int(m["id_bit"])) - 1) for r in raw]
            per_ctf[i] = np.bincount(np.array(vals, np.int64), minlength=n)
        checked = 0
        for oid in np.nonzero(res["sids"])[0][:4000]:
            sid = int(res["sids"][oid])
            want = int(o_count[oid]) if sid == 1 else int(per_ctf[sid - 2][oid])
            assert lib.ref_store_find(h, int(oid)) == want, (oid, sid)
            checked += 1
        assert checked > 100
    finally:
        lib.ref_store_free(h)
