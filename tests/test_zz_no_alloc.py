"""glint_active_search_noalloc against glint_active_search.

The allocation-free entry point takes device arrays and keeps its scratch in a
fixed device array of the library.  Two calls in a row (with different id
lists, so the second depends on the first having cleared its bitmap) must
return exactly what the allocating entry point returns, also when both are
enqueued on the stream with no host synchronisation between them, and a
call whose capacity is too small must report the full count, write only cap
records and leave the rest of the caller's buffer untouched.  This file is
named to be collected last, after every other GPU test has used the library.
"""
import ctypes
import glob

import numpy as np
import pytest

from glint_pipeline_gb300 import Configuration, DeviceBench, SEARCH_DTYPE, _abi
from workloads import case_config, make_points

pytestmark = pytest.mark.gpu


def _cudart():
    for cand in ["libcudart.so", "libcudart.so.13"] + glob.glob("/usr/local/cuda/lib64/libcudart.so*"):
        try:
            return ctypes.CDLL(cand)
        except OSError:
            continue
    raise OSError("libcudart not found")


class _Dev:
    """cudaMalloc'd test buffer (the caller's memory, not the library's)."""

    def __init__(self, rt, nbytes):
        self.rt = rt
        p = ctypes.c_void_p()
        assert rt.cudaMalloc(ctypes.byref(p), ctypes.c_size_t(max(nbytes, 1))) == 0
        self.ptr = p.value
        self.nbytes = nbytes

    def upload(self, arr):
        a = np.ascontiguousarray(arr)
        assert self.rt.cudaMemcpy(ctypes.c_void_p(self.ptr), a.ctypes.data_as(ctypes.c_void_p),
                                  ctypes.c_size_t(a.nbytes), 1) == 0

    def download(self, arr):
        assert self.rt.cudaMemcpy(arr.ctypes.data_as(ctypes.c_void_p), ctypes.c_void_p(self.ptr),
                                  ctypes.c_size_t(arr.nbytes), 2) == 0
        return arr

    def fill(self, byte):
        assert self.rt.cudaMemset(ctypes.c_void_p(self.ptr), byte, ctypes.c_size_t(self.nbytes)) == 0

    def free(self):
        self.rt.cudaFree(ctypes.c_void_p(self.ptr))


def test_noalloc_search_matches_allocating_search():
    box, pts = make_points("dense_20k", 24)
    cfgd = case_config("dense_20k")
    cfg = Configuration(num_objects=cfgd["num_objects"], grid_capacity=cfgd["grid_capacity"],
                        grid_amplify=cfgd["grid_amplify"], num_meeting_buckets=cfgd["num_meeting_buckets"],
                        reach_distance=cfgd["reach_distance"], min_meet_time=cfgd["min_meet_time"],
                        schema_update_delay=cfgd["schema_update_delay"])
    g = DeviceBench(cfg, box, pts[0])
    for t in range(pts.shape[0]):
        g.step(pts[t], t)
    lib = _abi.lib()
    rt = _cudart()
    rng = np.random.default_rng(5)
    n_obj = cfgd["num_objects"]
    lists = [rng.choice(n_obj, 3000, replace=False).astype(np.uint32),
             rng.choice(n_obj, 700, replace=False).astype(np.uint32)]
    cap = 20000
    d_pids = _Dev(rt, 4 * max(len(x) for x in lists))
    d_out = _Dev(rt, 32 * cap)
    d_n = _Dev(rt, 8)
    try:
        for pids in lists:
            want = g.active_search(pids)
            assert 0 < len(want) < cap
            d_pids.upload(pids)
            d_out.fill(0xAB)
            d_n.fill(0)
            st = lib.glint_active_search_noalloc(g.h, ctypes.c_void_p(d_pids.ptr), len(pids),
                                                 ctypes.c_void_p(d_out.ptr), cap, ctypes.c_void_p(d_n.ptr))
            assert st == 0, g.last_error()
            assert rt.cudaStreamSynchronize(ctypes.c_void_p(g.stream)) == 0
            n = int(d_n.download(np.zeros(1, np.uint64))[0])
            got = d_out.download(np.zeros(cap, SEARCH_DTYPE))[:n]
            assert n == len(want)
            assert got.tobytes() == want.tobytes()
        # truncation: the count is the full count, only cap records are
        # written, the sentinel bytes after them stay as they were
        pids = lists[0]
        want = g.active_search(pids)
        small = len(want) // 2
        d_pids.upload(pids)
        d_out.fill(0xAB)
        d_n.fill(0)
        st = lib.glint_active_search_noalloc(g.h, ctypes.c_void_p(d_pids.ptr), len(pids),
                                             ctypes.c_void_p(d_out.ptr), small, ctypes.c_void_p(d_n.ptr))
        assert st == 0, g.last_error()
        assert rt.cudaStreamSynchronize(ctypes.c_void_p(g.stream)) == 0
        assert int(d_n.download(np.zeros(1, np.uint64))[0]) == len(want)
        raw = d_out.download(np.zeros(32 * cap, np.uint8))
        assert raw[:32 * small].tobytes() == want[:small].tobytes()
        assert np.all(raw[32 * small:] == 0xAB)
        # two calls enqueued back to back on the context's stream, one host
        # synchronisation after both
        outs = [_Dev(rt, 32 * cap), _Dev(rt, 32 * cap)]
        ins = [_Dev(rt, 4 * len(x)) for x in lists]
        ns = [_Dev(rt, 8), _Dev(rt, 8)]
        try:
            for k, pids in enumerate(lists):
                ins[k].upload(pids)
                ns[k].fill(0)
            for k, pids in enumerate(lists):
                st = lib.glint_active_search_noalloc(g.h, ctypes.c_void_p(ins[k].ptr), len(pids),
                                                     ctypes.c_void_p(outs[k].ptr), cap, ctypes.c_void_p(ns[k].ptr))
                assert st == 0, g.last_error()
            assert rt.cudaStreamSynchronize(ctypes.c_void_p(g.stream)) == 0
            for k, pids in enumerate(lists):
                want = g.active_search(pids)
                n = int(ns[k].download(np.zeros(1, np.uint64))[0])
                assert n == len(want)
                assert outs[k].download(np.zeros(cap, SEARCH_DTYPE))[:n].tobytes() == want.tobytes()
        finally:
            for d in outs + ins + ns:
                d.free()
    finally:
        d_pids.free()
        d_out.free()
        d_n.free()
        g.close()
