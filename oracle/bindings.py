"""ctypes bindings for the test oracle (liboracle.so, the C restatement) and for
the reference's own CPU stages built into _ref/libglintref.so.

TEST INFRASTRUCTURE: imported only by tests/, __graft_entry__.smoke() and
bench.py's cpu_baseline leg.  The product never imports this module.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE_SO = os.path.join(HERE, "liboracle.so")
# GLINT_REF_SO selects another build of the reference's CPU stages (e.g. the
# as-shipped flags, build_ref.sh REF_OPT/REF_LIB)
REF_SO = os.environ.get("GLINT_REF_SO") or os.path.join(HERE, "_ref", "libglintref.so")
# the reference checkout: GLINT_REFERENCE_ROOT, else a directory named
# "reference" beside this repository
REFERENCE_ROOT = os.environ.get("GLINT_REFERENCE_ROOT") or os.path.join(os.path.dirname(os.path.dirname(HERE)),
                                                                          "reference")


def build_oracle() -> str:
    subprocess.run(["make", "-s", "-C", HERE, "liboracle.so"], check=True)
    return ORACLE_SO


REF_GPU_SO = os.path.join(HERE, "_ref", "libglintrefgpu.so")
REF_CUBIN = os.path.join(HERE, "_ref", "geometry.cubin")
REF_LAYOUT = os.path.join(HERE, "_ref", "ref_gpu_layout.h")


def build_ref_gpu() -> str | None:
    """Builds the driver that runs the reference's own GPU kernels
    (ref_gpu_driver.cpp) where build_ref.sh has left their cubin and layout
    header; returns None where they are absent."""
    if not (os.path.exists(REF_CUBIN) and os.path.exists(REF_LAYOUT)):
        return None
    src = os.path.join(HERE, "ref_gpu_driver.cpp")
    if os.path.exists(REF_GPU_SO) and os.path.getmtime(REF_GPU_SO) >= max(
            os.path.getmtime(src), os.path.getmtime(REF_LAYOUT), os.path.getmtime(ORACLE_SO)):
        return REF_GPU_SO
    cuda = os.environ.get("CUDA_HOME", "/usr/local/cuda")
    subprocess.run(["g++", "-std=c++17", "-O2", "-fPIC", "-shared", f"-I{HERE}", f"-I{cuda}/include", src,
                    "-o", REF_GPU_SO, f"-L{cuda}/lib64/stubs", f"-L{cuda}/lib64", "-lcuda", f"-L{HERE}", "-loracle",
                    "-Wl,-rpath," + HERE], check=True)
    return REF_GPU_SO


def ref_gpu_available() -> bool:
    return os.path.exists(REF_CUBIN) and os.path.exists(REF_LAYOUT)


def build_ref() -> str | None:
    """Builds the reference's own sources when they are present (this
    container); returns None elsewhere."""
    if not os.path.isdir(os.path.join(REFERENCE_ROOT, "src", "tracing")):
        return None
    subprocess.run(["sh", os.path.join(HERE, "build_ref.sh"), REFERENCE_ROOT], check=True,
                   stdout=subprocess.DEVNULL)
    return REF_SO


class GoConfig(ctypes.Structure):
    _fields_ = [
        ("num_objects", ctypes.c_uint32),
        ("grid_capacity", ctypes.c_uint32),
        ("schema_update_delay", ctypes.c_uint32),
        ("min_meet_time", ctypes.c_uint32),
        ("dynamic_schema", ctypes.c_uint32),
        ("pad0", ctypes.c_uint32),
        ("num_meeting_buckets", ctypes.c_uint64),
        ("grid_amplify", ctypes.c_double),
        ("reach_distance", ctypes.c_double),
    ]


class GoCounts(ctypes.Structure):
    _fields_ = [
        ("grid_check_counter", ctypes.c_uint32),
        ("kv_count", ctypes.c_uint32),
        ("num_taken_buckets", ctypes.c_uint64),
        ("num_active_meetings", ctypes.c_uint32),
        ("grids_stack_index", ctypes.c_uint32),
        ("schema_stack_index", ctypes.c_uint32),
        ("grids_stack_capacity", ctypes.c_uint32),
        ("schema_stack_capacity", ctypes.c_uint32),
        ("grid_capacity", ctypes.c_uint32),
        ("contacts", ctypes.c_uint64),
        ("candidates", ctypes.c_uint64),
        ("n_splits", ctypes.c_uint32),
        ("n_merges", ctypes.c_uint32),
        ("x_buffer", ctypes.c_double),
        ("y_buffer", ctypes.c_double),
        ("range_reruns", ctypes.c_uint32),
        ("pad1", ctypes.c_uint32),
    ]


MEETING_DTYPE = np.dtype([("key", "<u8"), ("start", "<u4"), ("end", "<u4"), ("mbr", "<f4", (4,))])
SCHEMA_DTYPE = np.dtype([
    ("grid_id", "<u4"), ("level", "<i2"), ("type", "<i2"), ("overflow_count", "<i2"),
    ("underflow_count", "<i2"), ("pad", "<u4"), ("mid_x", "<f8"), ("mid_y", "<f8"),
    ("low", "<f8", (2,)), ("high", "<f8", (2,)), ("children", "<u4", (4,)),
])
assert SCHEMA_DTYPE.itemsize == 80
# search_info_unit (tracing/workbench.h:85-88)
SEARCH_DTYPE = np.dtype([("pid", "<u4"), ("target", "<u4"), ("start", "<u4"), ("end", "<u4"), ("mbr", "<f4", (4,))])
assert SEARCH_DTYPE.itemsize == 32


# go_ctf_meta / glint_ctf_meta: CTF (tracing/step_merge.h) without its pointers
CTF_META_DTYPE = np.dtype([("ctf_mbr", "<f4", (4,)), ("CTF_kv_capacity", "<u4"), ("start_time_min", "<u4"),
                           ("start_time_max", "<u4"), ("end_time_min", "<u4"), ("end_time_max", "<u4"),
                           ("ctf_bitmap_size", "<u4"), ("key_bit", "<u2"), ("id_bit", "<u2"),
                           ("duration_bit", "<u2"), ("end_bit", "<u2"), ("low_x_bit", "<u2"), ("low_y_bit", "<u2"),
                           ("edge_bit", "<u2"), ("mbr_bit", "<u2"), ("x_grid", "<u2"), ("y_grid", "<u2"),
                           ("reserved", "<u4")])
assert CTF_META_DTYPE.itemsize == 64
BIT_BYTES = 256 * 256 // 8


class GoStoreConfig(ctypes.Structure):
    _fields_ = [("num_objects", ctypes.c_uint32), ("max_meet_time", ctypes.c_uint32), ("CTF_count", ctypes.c_uint32),
                ("split_num", ctypes.c_uint32), ("first_end_time_min", ctypes.c_uint32), ("pad0", ctypes.c_uint32),
                ("dProbFalse", ctypes.c_double), ("mbr", ctypes.c_double * 4), ("kv_capacity", ctypes.c_uint64)]


class StoreInfo(ctypes.Structure):
    """go_store_info / glint_store_info"""
    _fields_ = [("kv_count", ctypes.c_uint64), ("key_bytes", ctypes.c_uint64), ("oversize_kv_count", ctypes.c_uint32),
                ("oversize_start_time_min", ctypes.c_uint32), ("oversize_start_time_max", ctypes.c_uint32),
                ("oversize_end_time_min", ctypes.c_uint32), ("oversize_end_time_max", ctypes.c_uint32),
                ("sid_count", ctypes.c_uint32), ("oversize_oid_count", ctypes.c_uint32),
                ("end_time_min", ctypes.c_uint32), ("cur_time", ctypes.c_uint32), ("reserved", ctypes.c_uint32),
                ("bits_outside", ctypes.c_uint64)]

    def as_dict(self):
        return {f: getattr(self, f) for f, _ in self._fields_ if f != "reserved"}


def _load_oracle():
    build_oracle()  # make: a no-op unless a source is newer than the library
    lib = ctypes.CDLL(ORACLE_SO)
    vp = ctypes.c_void_p
    lib.go_create.restype = vp
    lib.go_create.argtypes = [ctypes.POINTER(GoConfig), vp, vp]
    lib.go_create_threads.restype = vp
    lib.go_create_threads.argtypes = [ctypes.POINTER(GoConfig), vp, vp, ctypes.c_uint32]
    lib.go_set_threads.argtypes = [vp, ctypes.c_uint32]
    lib.go_destroy.argtypes = [vp]
    lib.go_step.argtypes = [vp, vp, ctypes.c_uint32]
    lib.go_get_counts.argtypes = [vp, ctypes.POINTER(GoCounts)]
    lib.go_get_meetings.restype = ctypes.c_uint32
    lib.go_get_meetings.argtypes = [vp, vp, ctypes.c_uint32]
    lib.go_get_schema.argtypes = [vp, vp, vp, vp, vp]
    lib.go_get_buckets.argtypes = [vp, vp, vp, vp, vp]
    lib.go_active_search.restype = ctypes.c_uint64
    lib.go_active_search.argtypes = [vp, vp, ctypes.c_uint32, vp, ctypes.c_uint64]
    lib.go_store_create.restype = vp
    lib.go_store_create.argtypes = [ctypes.POINTER(GoStoreConfig)]
    lib.go_store_destroy.argtypes = [vp]
    lib.go_store_add_meetings.argtypes = [vp, vp, ctypes.c_uint64]
    lib.go_store_kv_count.restype = ctypes.c_uint64
    lib.go_store_kv_count.argtypes = [vp]
    lib.go_store_flush.restype = ctypes.c_int
    lib.go_store_flush.argtypes = [vp, ctypes.c_uint32, ctypes.POINTER(StoreInfo)]
    lib.go_store_result.argtypes = [vp] * 9
    lib.go_store_sorted.restype = ctypes.c_uint64
    lib.go_store_sorted.argtypes = [vp, vp, vp]
    lib.go_query_bfs.restype = ctypes.c_uint64
    lib.go_query_bfs.argtypes = [vp, ctypes.c_uint64, ctypes.c_uint32, vp, ctypes.c_uint32, ctypes.c_uint32,
                                 ctypes.c_uint32, ctypes.c_uint32, vp, ctypes.c_uint64, vp]
    lib.go_dpm_lon.restype = ctypes.c_double
    lib.go_dpm_lon.argtypes = [ctypes.c_double]
    lib.go_sin_cr.restype = ctypes.c_double
    lib.go_sin_cr.argtypes = [ctypes.c_double]
    lib.go_cantor.restype = ctypes.c_uint64
    lib.go_cantor.argtypes = [ctypes.c_uint32, ctypes.c_uint32]
    lib.go_compact.restype = ctypes.c_int
    lib.go_compact.argtypes = [vp, ctypes.c_uint32, ctypes.c_uint32, vp, ctypes.c_uint32, ctypes.c_uint32,
                               ctypes.c_int, ctypes.POINTER(vp)]
    lib.go_compact_sizes.argtypes = [vp, vp]
    lib.go_compact_result.argtypes = [vp] * 9
    lib.go_compact_free.argtypes = [vp]
    return lib


_ORACLE = None


def oracle_lib():
    global _ORACLE
    if _ORACLE is None:
        _ORACLE = _load_oracle()
    return _ORACLE


def make_config(num_objects, *, grid_capacity=50, schema_update_delay=1, min_meet_time=5, dynamic_schema=True,
                num_meeting_buckets=None, grid_amplify=2.0, reach_distance=2.0) -> GoConfig:
    return GoConfig(num_objects, grid_capacity, schema_update_delay, min_meet_time, int(bool(dynamic_schema)), 0,
                    int(num_meeting_buckets if num_meeting_buckets is not None else 2 * num_objects),
                    float(grid_amplify), float(reach_distance))


class Oracle:
    """CPU restatement of the reference's per-step stages.  threads > 1 runs
    the order-free parts on host threads; the results are those of one
    thread."""

    def __init__(self, cfg: GoConfig, mbr: np.ndarray, first_points: np.ndarray, threads: int = 1):
        self.lib = oracle_lib()
        self.cfg = cfg
        self._mbr = np.ascontiguousarray(mbr, dtype=np.float64)
        pts = np.ascontiguousarray(first_points, dtype=np.float64)
        self.h = self.lib.go_create_threads(ctypes.byref(cfg), self._mbr.ctypes.data, pts.ctypes.data,
                                            max(1, int(threads)))
        if not self.h:
            raise MemoryError("go_create failed")

    def step(self, points: np.ndarray, cur_time: int):
        pts = np.ascontiguousarray(points, dtype=np.float64)
        self.lib.go_step(self.h, pts.ctypes.data, int(cur_time))

    def counts(self) -> GoCounts:
        c = GoCounts()
        self.lib.go_get_counts(self.h, ctypes.byref(c))
        return c

    def meetings(self) -> np.ndarray:
        c = self.counts()
        out = np.zeros(max(c.kv_count, 1), dtype=MEETING_DTYPE)
        n = self.lib.go_get_meetings(self.h, out.ctypes.data, out.shape[0])
        return out[: min(n, out.shape[0])]

    def schema(self):
        c = self.counts()
        sch = np.zeros(c.schema_stack_capacity, dtype=SCHEMA_DTYPE)
        ss = np.zeros(c.schema_stack_capacity, dtype=np.uint32)
        gs = np.zeros(c.grids_stack_capacity, dtype=np.uint32)
        gc = np.zeros(c.grids_stack_capacity, dtype=np.uint32)
        self.lib.go_get_schema(self.h, sch.ctypes.data, ss.ctypes.data, gs.ctypes.data, gc.ctypes.data)
        return sch, ss, gs, gc

    def buckets(self):
        B = int(self.cfg.num_meeting_buckets)
        k = np.zeros(B, np.uint64)
        s = np.zeros(B, np.uint32)
        e = np.zeros(B, np.uint32)
        m = np.zeros((B, 4), np.float32)
        self.lib.go_get_buckets(self.h, k.ctypes.data, s.ctypes.data, e.ctypes.data, m.ctypes.data)
        return k, s, e, m

    def active_search(self, pids) -> np.ndarray:
        """Active meetings of the listed objects after the last step
        (cuda/geometry.cu:605-663), in bucket order."""
        p = np.ascontiguousarray(pids, dtype=np.uint32)
        n = self.lib.go_active_search(self.h, p.ctypes.data, p.shape[0], None, 0)
        out = np.zeros(max(int(n), 1), dtype=SEARCH_DTYPE)
        self.lib.go_active_search(self.h, p.ctypes.data, p.shape[0], out.ctypes.data, out.shape[0])
        return out[: int(n)]

    def close(self):
        if self.h:
            self.lib.go_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


EDGE_DTYPE = np.dtype([("pid", "<u4"), ("target", "<u4"), ("start", "<u4"), ("end", "<u4")])


def query_bfs(edges: np.ndarray, num_objects: int, seeds, hops: int, t_start: int = 0, t_end: int = 0):
    """Contact-trace BFS over store edges (glint_query_oracle.c): a list of
    per-hop arrays of newly reached object ids (ascending)."""
    lib = oracle_lib()
    e = np.ascontiguousarray(edges, dtype=EDGE_DTYPE)
    sd = np.ascontiguousarray(seeds, dtype=np.uint32)
    hop_end = np.zeros(max(hops, 1), np.uint64)
    n = lib.go_query_bfs(e.ctypes.data, e.shape[0], num_objects, sd.ctypes.data, sd.shape[0], t_start, t_end, hops,
                         None, 0, hop_end.ctypes.data)
    out = np.zeros(max(int(n), 1), np.uint32)
    lib.go_query_bfs(e.ctypes.data, e.shape[0], num_objects, sd.ctypes.data, sd.shape[0], t_start, t_end, hops,
                     out.ctypes.data, out.shape[0], hop_end.ctypes.data)
    bounds = [0] + [int(v) for v in hop_end[:hops]]
    return [out[bounds[h]:bounds[h + 1]] for h in range(hops)]


class GoBlock(ctypes.Structure):
    """go_block: one source block of a compaction"""
    _fields_ = [("CTF_count", ctypes.c_uint32), ("o_count", ctypes.c_uint32), ("sids", ctypes.c_void_p),
                ("ctfs", ctypes.c_void_p), ("keys", ctypes.c_void_p), ("o_keys", ctypes.c_void_p),
                ("o_boxes", ctypes.c_void_p), ("o_bitmap", ctypes.c_void_p), ("o_times", ctypes.c_uint32 * 4),
                ("times", ctypes.c_uint32 * 4)]


COMPACT_ERRORS = {-1: "no object has a CTF key", -2: "too few objects for split_num",
                  -3: "an object id beyond num_objects", -4: "get_ctf_bits out of domain"}


def compact_blocks(blocks, num_objects, mbr, split_num, max_meet_time=4096, std_ties=False):
    """CPU restatement of the reference's merge_dump (glint_compact_oracle.c).

    blocks: dicts with keys, sids, ctfs, o_keys, o_boxes, o_bitmap, o_times
    (4) and times (4), as Store.result / the device store give them.
    std_ties: equivalent elements in the order of the C++ library's std::sort
    (the reference's exact output) instead of a stable order (the device's).
    Returns (rc, result dict or None)."""
    lib = oracle_lib()
    keep = []
    arr = (GoBlock * len(blocks))()
    for i, b in enumerate(blocks):
        fields = {}
        for k in ("sids", "ctfs", "keys", "o_keys", "o_boxes", "o_bitmap"):
            a = np.ascontiguousarray(b[k])
            if a.size == 0:
                a = np.zeros(16, np.uint8)
            keep.append(a)
            fields[k] = a.ctypes.data
        arr[i] = GoBlock(len(b["ctfs"]), len(b["o_keys"]), fields["sids"], fields["ctfs"], fields["keys"],
                         fields["o_keys"], fields["o_boxes"], fields["o_bitmap"],
                         (ctypes.c_uint32 * 4)(*[int(v) for v in b["o_times"]]),
                         (ctypes.c_uint32 * 4)(*[int(v) for v in b.get("times", (0, 0, 0, 0))]))
    m = np.ascontiguousarray(mbr, dtype=np.float64)
    h = ctypes.c_void_p()
    rc = lib.go_compact(ctypes.cast(arr, ctypes.c_void_p), len(blocks), int(num_objects), m.ctypes.data,
                        int(max_meet_time), int(split_num), int(bool(std_ties)), ctypes.byref(h))
    if rc != 0:
        return rc, None
    try:
        sizes = np.zeros(8, np.uint64)
        lib.go_compact_sizes(h, sizes.ctypes.data)
        C, kv, kb, on = (int(v) for v in sizes[:4])
        out = {"keys": np.zeros(kb, np.uint8), "sids": np.zeros(int(num_objects), np.uint16),
               "ctfs": np.zeros(C, CTF_META_DTYPE), "bitmaps": np.zeros(C * BIT_BYTES, np.uint8),
               "o_keys": np.zeros((on, 16), np.uint8), "o_boxes": np.zeros((on, 4), np.float32),
               "o_bitmap": np.zeros(BIT_BYTES, np.uint8), "times8": np.zeros(8, np.uint32)}
        lib.go_compact_result(h, *[out[k].ctypes.data for k in
                                   ("keys", "sids", "ctfs", "bitmaps", "o_keys", "o_boxes", "o_bitmap", "times8")])
        out.update(kv_count=kv, key_bytes=kb, o_count=on, padding=int(sizes[4]), x_part=int(sizes[5]),
                   y_part=int(sizes[6]), sid_count=int(sizes[7]))
        return 0, out
    finally:
        lib.go_compact_free(h)


class Store:
    """CPU restatement of the GPU path's key generation and flush
    (glint_flush_oracle.c)."""

    def __init__(self, num_objects, mbr, *, max_meet_time=4096, CTF_count=100, split_num=10, first_end_time_min=5,
                 dProbFalse=100.0, kv_capacity=1 << 22):
        self.lib = oracle_lib()
        self.cfg = GoStoreConfig(num_objects, max_meet_time, CTF_count, split_num, first_end_time_min, 0,
                                 float(dProbFalse), (ctypes.c_double * 4)(*[float(v) for v in mbr]), int(kv_capacity))
        self.h = self.lib.go_store_create(ctypes.byref(self.cfg))

    def add_meetings(self, meetings: np.ndarray):
        """meetings: records (pid1, pid2, start, end, mbr[4]) of one step"""
        m = np.ascontiguousarray(meetings)
        assert m.dtype.itemsize == 32
        self.lib.go_store_add_meetings(self.h, m.ctypes.data, m.shape[0])

    @property
    def kv_count(self) -> int:
        return int(self.lib.go_store_kv_count(self.h))

    def flush(self, cur_time: int):
        info = StoreInfo()
        rc = self.lib.go_store_flush(self.h, int(cur_time), ctypes.byref(info))
        return rc, info

    def result(self, info: StoreInfo) -> dict:
        C, N = self.cfg.CTF_count, self.cfg.num_objects
        out = {"keys": np.zeros(int(info.key_bytes), np.uint8), "sids": np.zeros(N, np.uint16),
               "ctf_capacity": np.zeros(C, np.uint32), "ctfs": np.zeros(C, CTF_META_DTYPE),
               "bitmaps": np.zeros(C * BIT_BYTES, np.uint8),
               "o_keys": np.zeros((int(info.oversize_kv_count), 16), np.uint8),
               "o_boxes": np.zeros((int(info.oversize_kv_count), 4), np.float32),
               "o_bitmap": np.zeros(BIT_BYTES, np.uint8)}
        self.lib.go_store_result(self.h, *[out[k].ctypes.data for k in
                                           ("keys", "sids", "ctf_capacity", "ctfs", "bitmaps", "o_keys", "o_boxes",
                                            "o_bitmap")])
        return out

    def sorted_keys(self, info: StoreInfo):
        """(keys as (n, 16) little-endian bytes, boxes (n, 4)) of the last flush"""
        n = int(info.kv_count) + int(info.oversize_kv_count)
        k = np.zeros((n, 16), np.uint8)
        b = np.zeros((n, 4), np.float32)
        self.lib.go_store_sorted(self.h, k.ctypes.data, b.ctypes.data)
        return k, b

    def close(self):
        if self.h:
            self.lib.go_store_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class RefConfig(ctypes.Structure):
    _fields_ = [
        ("num_objects", ctypes.c_uint32), ("num_threads", ctypes.c_uint32), ("grid_capacity", ctypes.c_uint32),
        ("schema_update_delay", ctypes.c_uint32), ("min_meet_time", ctypes.c_uint32),
        ("dynamic_schema", ctypes.c_uint32), ("num_meeting_buckets", ctypes.c_uint64),
        ("grid_amplify", ctypes.c_double), ("reach_distance", ctypes.c_double),
        ("start_time", ctypes.c_uint32), ("pad", ctypes.c_uint32),
    ]


class RefCounts(ctypes.Structure):
    _fields_ = [
        ("grid_check_counter", ctypes.c_uint32), ("kv_count", ctypes.c_uint32),
        ("num_taken_buckets", ctypes.c_uint64), ("num_active_meetings", ctypes.c_uint32),
        ("grids_stack_index", ctypes.c_uint32), ("schema_stack_index", ctypes.c_uint32),
        ("grids_stack_capacity", ctypes.c_uint32), ("schema_stack_capacity", ctypes.c_uint32),
        ("grid_capacity", ctypes.c_uint32), ("x_buffer", ctypes.c_double), ("y_buffer", ctypes.c_double),
        ("ms_filter", ctypes.c_double), ("ms_refine", ctypes.c_double), ("ms_meet", ctypes.c_double),
        ("ms_schema", ctypes.c_double),
    ]


_REF = None


def ref_available() -> bool:
    return os.path.exists(REF_SO) or os.path.isdir(os.path.join(REFERENCE_ROOT, "src", "tracing"))


def ref_lib():
    global _REF
    if _REF is None:
        driver = os.path.join(HERE, "ref_driver.cpp")
        if not os.path.exists(REF_SO) or os.path.getmtime(driver) > os.path.getmtime(REF_SO):
            if build_ref() is None:
                raise FileNotFoundError("reference build unavailable (no sources on this machine)")
        lib = ctypes.CDLL(REF_SO)
        vp = ctypes.c_void_p
        lib.ref_create.restype = vp
        lib.ref_create.argtypes = [ctypes.POINTER(RefConfig), vp, vp]
        lib.ref_step.argtypes = [vp, vp, ctypes.c_uint32]
        lib.ref_get_counts.argtypes = [vp, ctypes.POINTER(RefCounts)]
        lib.ref_get_meetings.restype = ctypes.c_uint32
        lib.ref_get_meetings.argtypes = [vp, vp, vp, vp, ctypes.c_uint32]
        lib.ref_get_schema.argtypes = [vp, vp, vp, vp, vp]
        lib.ref_get_buckets.argtypes = [vp, vp, vp, vp]
        lib.ref_schema_record_size.restype = ctypes.c_uint32
        lib.ref_dpm_lon.restype = ctypes.c_double
        lib.ref_dpm_lon.argtypes = [ctypes.c_double]
        lib.ref_destroy.argtypes = [vp]
        lib.ref_ctf_bits.argtypes = [vp, vp, ctypes.c_uint32, ctypes.c_uint32, vp, vp]
        lib.ref_serial_mbr.restype = ctypes.c_uint64
        lib.ref_serial_mbr.argtypes = [vp, vp, vp]
        lib.ref_serial_key.argtypes = [vp, vp, ctypes.c_uint64, ctypes.c_uint64, ctypes.c_uint64, ctypes.c_uint64,
                                       ctypes.c_uint64, vp]
        lib.ref_ctf_find.restype = ctypes.c_int
        lib.ref_ctf_find.argtypes = [vp, vp, vp, ctypes.c_uint32, ctypes.c_uint32, ctypes.POINTER(ctypes.c_uint32)]
        lib.ref_store_load.restype = vp
        lib.ref_store_load.argtypes = [ctypes.c_char_p, ctypes.c_char_p, ctypes.c_char_p, ctypes.c_uint32,
                                       ctypes.c_uint32, ctypes.c_uint32]
        lib.ref_store_get.argtypes = [vp] * 9
        lib.ref_store_find.restype = ctypes.c_uint32
        lib.ref_store_find.argtypes = [vp, ctypes.c_uint32]
        lib.ref_store_free.argtypes = [vp]
        lib.ref_compact.restype = ctypes.c_int
        lib.ref_compact.argtypes = [ctypes.c_char_p, ctypes.c_char_p, ctypes.c_char_p, ctypes.c_uint32,
                                    ctypes.c_uint32, ctypes.c_uint32, vp, ctypes.c_uint32, ctypes.c_uint32,
                                    ctypes.c_char_p]
        _REF = lib
    return _REF


class Reference:
    """The reference's own CPU stages (tracing/*.cpp), one step at a time."""

    def __init__(self, cfg: GoConfig, mbr: np.ndarray, first_points: np.ndarray, num_threads: int = 1,
                 start_time: int = 0):
        self.lib = ref_lib()
        self.cfg = cfg
        rc = RefConfig(cfg.num_objects, num_threads, cfg.grid_capacity, cfg.schema_update_delay, cfg.min_meet_time,
                       cfg.dynamic_schema, cfg.num_meeting_buckets, cfg.grid_amplify, cfg.reach_distance,
                       start_time, 0)
        self._mbr = np.ascontiguousarray(mbr, dtype=np.float64)
        pts = np.ascontiguousarray(first_points, dtype=np.float64)
        self.h = self.lib.ref_create(ctypes.byref(rc), self._mbr.ctypes.data, pts.ctypes.data)

    def step(self, points: np.ndarray, cur_time: int):
        pts = np.ascontiguousarray(points, dtype=np.float64)
        self.lib.ref_step(self.h, pts.ctypes.data, int(cur_time))

    def counts(self) -> RefCounts:
        c = RefCounts()
        self.lib.ref_get_counts(self.h, ctypes.byref(c))
        return c

    def meetings(self) -> np.ndarray:
        c = self.counts()
        n = max(c.kv_count, 1)
        k = np.zeros(n, np.uint64)
        s = np.zeros(n, np.uint32)
        e = np.zeros(n, np.uint32)
        got = self.lib.ref_get_meetings(self.h, k.ctypes.data, s.ctypes.data, e.ctypes.data, n)
        got = min(got, n)
        out = np.zeros(got, dtype=MEETING_DTYPE)
        out["key"] = k[:got]
        out["start"] = s[:got]
        out["end"] = e[:got]
        return out

    def schema(self):
        c = self.counts()
        assert self.lib.ref_schema_record_size() == 80
        sch = np.zeros(c.schema_stack_capacity, dtype=SCHEMA_DTYPE)
        ss = np.zeros(c.schema_stack_capacity, dtype=np.uint32)
        gs = np.zeros(c.grids_stack_capacity, dtype=np.uint32)
        gc = np.zeros(c.grids_stack_capacity, dtype=np.uint32)
        self.lib.ref_get_schema(self.h, sch.ctypes.data, ss.ctypes.data, gs.ctypes.data, gc.ctypes.data)
        return sch, ss, gs, gc

    def buckets(self):
        B = int(self.cfg.num_meeting_buckets)
        k = np.zeros(B, np.uint64)
        s = np.zeros(B, np.uint32)
        e = np.zeros(B, np.uint32)
        self.lib.ref_get_buckets(self.h, k.ctypes.data, s.ctypes.data, e.ctypes.data)
        return k, s, e

    def close(self):
        if self.h:
            self.lib.ref_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def cantor_inverse(keys: np.ndarray):
    """Exact (a, b) with key = (a+b)(a+b+1)/2 + b, vectorised."""
    z = keys.astype(np.uint64)
    w = np.floor((np.sqrt(8.0 * z.astype(np.float64) + 1) - 1) / 2).astype(np.uint64)
    for _ in range(3):
        over = w * (w + np.uint64(1)) // np.uint64(2) > z
        w = np.where(over, w - np.uint64(1), w)
        under = (w + np.uint64(1)) * (w + np.uint64(2)) // np.uint64(2) <= z
        w = np.where(under, w + np.uint64(1), w)
    t = w * (w + np.uint64(1)) // np.uint64(2)
    b = (z - t).astype(np.uint64)
    a = (w - b).astype(np.uint64)
    return a.astype(np.uint32), b.astype(np.uint32)


class RgConfig(ctypes.Structure):
    _fields_ = [("device", ctypes.c_uint32), ("num_objects", ctypes.c_uint32), ("CTF_count", ctypes.c_uint32),
                ("split_num", ctypes.c_uint32), ("min_meet_time", ctypes.c_uint32),
                ("max_meet_time", ctypes.c_uint32), ("kv_capacity", ctypes.c_uint64), ("dProbFalse", ctypes.c_double),
                ("mbr", ctypes.c_double * 4)]


class RgFlushInfo(ctypes.Structure):
    _fields_ = [("kv_count", ctypes.c_uint64), ("key_bytes", ctypes.c_uint64), ("oversize_kv_count", ctypes.c_uint32),
                ("oversize_start_time_min", ctypes.c_uint32), ("oversize_start_time_max", ctypes.c_uint32),
                ("oversize_end_time_min", ctypes.c_uint32), ("oversize_end_time_max", ctypes.c_uint32),
                ("sid_count", ctypes.c_uint32), ("oversize_oid_count", ctypes.c_uint32), ("pad", ctypes.c_uint32),
                ("bits_in_slack", ctypes.c_uint64)]


class RefGpu:
    """The reference's own GPU kernels (cuda/geometry.cu, compiled unmodified
    into oracle/_ref/geometry.cubin) driven as process_with_gpu drives them:
    key generation and the active multi-search by cuda_identify_meetings,
    and the flush into the key-value + bitmap store.  Needs a GPU."""

    def __init__(self, num_objects, mbr, *, CTF_count=100, split_num=10, min_meet_time=5, max_meet_time=4096,
                 kv_capacity=1 << 22, dProbFalse=100.0, device=0):
        build_oracle()
        so = build_ref_gpu()
        if so is None:
            raise RuntimeError("the reference's GPU kernels are not built here (oracle/build_ref.sh)")
        self.lib = lib = ctypes.CDLL(so)
        vp = ctypes.c_void_p
        lib.rg_open.argtypes = [ctypes.c_char_p, ctypes.POINTER(RgConfig), ctypes.POINTER(vp)]
        lib.rg_error.restype = ctypes.c_char_p
        lib.rg_error.argtypes = [vp]
        lib.rg_identify.argtypes = [vp, vp, ctypes.c_uint64, ctypes.c_uint32, ctypes.c_uint32, vp, ctypes.c_uint32,
                                    vp, ctypes.c_uint64, ctypes.POINTER(ctypes.c_uint64)]
        lib.rg_pending.argtypes = [vp, ctypes.POINTER(ctypes.c_uint64), ctypes.POINTER(ctypes.c_uint32),
                                   ctypes.POINTER(ctypes.c_uint32)]
        lib.rg_flush.argtypes = [vp, ctypes.c_uint32, ctypes.POINTER(RgFlushInfo)]
        lib.rg_result.argtypes = [vp] * 9
        lib.rg_close.argtypes = [vp]
        self.n, self.C = int(num_objects), int(CTF_count)
        cfg = RgConfig(device, self.n, self.C, split_num, min_meet_time, max_meet_time, kv_capacity, dProbFalse,
                       (ctypes.c_double * 4)(*[float(v) for v in mbr]))
        self.h = vp()
        rc = lib.rg_open(REF_CUBIN.encode(), ctypes.byref(cfg), ctypes.byref(self.h))
        if rc != 0:
            msg = lib.rg_error(self.h).decode()
            self.close()
            raise RuntimeError(f"rg_open: {msg}")

    def _check(self, rc, what):
        if rc != 0:
            raise RuntimeError(f"{what} ({rc}): {self.lib.rg_error(self.h).decode()}")

    def identify(self, meetings, cur_time, end_time_min, pids=None):
        """meetings: MEETING_DTYPE records (Cantor key, start, end, f32 box),
        the layout of meeting_unit; pids: the multi-search list, or None.
        Returns the multi-search's records (in the reference's atomic
        order)."""
        m = np.ascontiguousarray(meetings, dtype=MEETING_DTYPE)
        p = np.ascontiguousarray(pids if pids is not None else np.zeros(0), dtype=np.uint32)
        found = ctypes.c_uint64()
        cap = 2 * max(1, m.shape[0]) * max(1, int(np.bincount(p).max()) if p.size else 1)
        out = np.zeros(cap if p.size else 1, SEARCH_DTYPE)
        rc = self.lib.rg_identify(self.h, m.ctypes.data if m.size else None, m.shape[0], int(cur_time),
                                  int(end_time_min), p.ctypes.data if p.size else None, p.shape[0], out.ctypes.data,
                                  out.shape[0], ctypes.byref(found))
        self._check(rc, "rg_identify")
        return out[: int(found.value)]

    def pending(self):
        kv, sc, oc = ctypes.c_uint64(), ctypes.c_uint32(), ctypes.c_uint32()
        self._check(self.lib.rg_pending(self.h, ctypes.byref(kv), ctypes.byref(sc), ctypes.byref(oc)), "rg_pending")
        return int(kv.value), int(sc.value), int(oc.value)

    def flush(self, cur_time):
        info = RgFlushInfo()
        self._check(self.lib.rg_flush(self.h, int(cur_time), ctypes.byref(info)), "rg_flush")
        r = {"info": info, "keys": np.zeros(int(info.key_bytes), np.uint8), "sids": np.zeros(self.n, np.uint16),
             "ctf_capacity": np.zeros(self.C, np.uint32), "ctfs": np.zeros(self.C, CTF_META_DTYPE),
             "bitmaps": np.zeros(self.C * BIT_BYTES, np.uint8),
             "o_keys": np.zeros(int(info.oversize_kv_count) * 16, np.uint8),
             "o_boxes": np.zeros((int(info.oversize_kv_count), 4), np.float32),
             "o_bitmap": np.zeros(BIT_BYTES, np.uint8)}
        self.lib.rg_result(self.h, *[r[k].ctypes.data for k in ("keys", "sids", "ctf_capacity", "ctfs", "bitmaps",
                                                               "o_keys", "o_boxes", "o_bitmap")])
        return r

    def close(self):
        if getattr(self, "h", None) and self.h.value:
            self.lib.rg_close(self.h)
            self.h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
