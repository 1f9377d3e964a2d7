"""GB300-native GLINT contact-tracing step.

Python mirror of the reference's GPU seam (tracing/process.cpp:373-376):

    bench = cuda_create_device_bench(config, mbr, first_points)   # geometry.cu:1395
    for t ...:
        stats = process_with_gpu(bench, points_t, cur_time=t)      # geometry.cu:1573
        meetings = bench.meetings()                                # meeting.cpp:147-153

Everything runs in libglint.so (hand-written sm_103a CUDA behind the C ABI in
include/glint.h).  There is no CPU fallback: constructing a DeviceBench
raises when the library is missing or no GPU is visible.
"""
from __future__ import annotations

import ctypes
import dataclasses
import os

import numpy as np

from . import _abi
from ._abi import GlintConfig, GlintStepStats, MEETING_DTYPE, SCHEMA_DTYPE, SEARCH_DTYPE, GlintError

__all__ = [
    "Configuration", "DeviceBench", "cuda_create_device_bench", "process_with_gpu", "GlintError",
    "MEETING_DTYPE", "SCHEMA_DTYPE", "SEARCH_DTYPE", "library_path", "load_library",
]

library_path = _abi.library_path
load_library = _abi.load_library


@dataclasses.dataclass
class Configuration:
    """The fields of the reference's `configuration` (util/config.h:15-114)
    that this path reads, with the reference's defaults."""
    num_objects: int = 1000
    grid_capacity: int = 50
    grid_amplify: float = 2.0
    num_meeting_buckets: int = 0        # 0 -> 2 * num_objects (config.h:176-178)
    reach_distance: float = 2.0
    min_meet_time: int = 5
    max_meet_time: int = 4096
    schema_update_delay: int = 1
    dynamic_schema: bool = True
    phased_lookup: bool = True
    start_time: int = 0
    x_buffer: float = 0.0
    y_buffer: float = 0.0
    G_bytes: int = 2
    CTF_count: int = 100
    dProbFalse: float = 100.0
    # this implementation
    precision_mode: int = 0             # 0 plain FP64, 1 FP32 guard band
    device: int = 0
    new_capacity: int = 0
    check_capacity: int = 0
    meeting_log_capacity: int = 0
    timing: bool = False
    auto_flush: bool = False
    split_num: int = 10
    store_keep: int = 16                # flushed blocks kept on the device for queries
    store_host_keep: int = 0            # further blocks kept in page-locked host memory for queries
    refine_chunk: int = 0               # cross-leaf checks per refine work item; 0 -> 64
    use_graph: bool = False             # capture the step as a CUDA graph
    kv_restriction: int = 0             # 0 -> G_bytes * 2^25 keys (config.h:80)
    kv_capacity: int = 0                # 0 -> kv_restriction + max(1e6, 4 N)

    def to_c(self) -> GlintConfig:
        c = GlintConfig()
        _abi.lib().glint_config_defaults(ctypes.byref(c), int(self.num_objects))
        for f in dataclasses.fields(self):
            v = getattr(self, f.name)
            if isinstance(v, bool):
                v = int(v)
            setattr(c, f.name, v)
        if not self.num_meeting_buckets:
            c.num_meeting_buckets = 2 * int(self.num_objects)
        return c


class DeviceBench:
    """Device-resident workbench: schema, leaf tiles, meeting table, meeting log."""

    def __init__(self, config: Configuration, mbr, first_points=None, schema=None):
        self.lib = _abi.lib()
        self.config = config
        self.n = int(config.num_objects)
        self._cfg = config.to_c()
        box = _abi.GlintBox()
        m = np.asarray(mbr, dtype=np.float64).reshape(4)
        box.low[0], box.low[1], box.high[0], box.high[1] = m
        self._box = box
        pts_ptr = None
        if first_points is not None:
            self._first = np.ascontiguousarray(first_points, dtype=np.float64).reshape(self.n, 2)
            pts_ptr = self._first.ctypes.data_as(ctypes.c_void_p)
        init_ptr = None
        if schema is not None:
            init_ptr = ctypes.byref(schema)
        h = ctypes.c_void_p()
        st = self.lib.glint_create(ctypes.byref(self._cfg), ctypes.byref(box), pts_ptr, init_ptr, ctypes.byref(h))
        if st != 0:
            raise GlintError(st, "glint_create")
        self.h = h
        sc = ctypes.c_uint32()
        gc = ctypes.c_uint32()
        bk = ctypes.c_uint64()
        self.lib.glint_get_capacities(self.h, ctypes.byref(sc), ctypes.byref(gc), ctypes.byref(bk))
        self.schema_capacity, self.grids_capacity, self.num_buckets = sc.value, gc.value, bk.value
        self._staging = None

    # -- per step -----------------------------------------------------------
    def step(self, points, cur_time: int) -> GlintStepStats:
        """process_with_gpu: host points in, synchronous."""
        pts = np.ascontiguousarray(points, dtype=np.float64)
        if pts.size != 2 * self.n:
            raise ValueError("points must hold num_objects (lon, lat) pairs")
        stats = GlintStepStats()
        st = self.lib.glint_step(self.h, pts.ctypes.data_as(ctypes.c_void_p), int(cur_time), ctypes.byref(stats))
        if st != 0:
            raise GlintError(st, self.last_error())
        return stats

    def step_device(self, d_points_ptr: int, cur_time: int):
        st = self.lib.glint_step_device(self.h, ctypes.c_void_p(int(d_points_ptr)), int(cur_time))
        if st != 0:
            raise GlintError(st, self.last_error())

    def sync(self) -> GlintStepStats:
        stats = GlintStepStats()
        st = self.lib.glint_sync(self.h, ctypes.byref(stats))
        if st != 0:
            raise GlintError(st, self.last_error())
        return stats

    def meetings(self, out: np.ndarray | None = None) -> np.ndarray:
        """Meetings identified by the last step, in bucket order.  With `out`
        (MEETING_DTYPE records, e.g. from pinned_empty) large enough, they
        are copied into it and out[:n] is returned; otherwise into a new
        array."""
        n = ctypes.c_uint64()
        st = self.lib.glint_meetings(self.h, None, 0, ctypes.byref(n))
        if st != 0:
            raise GlintError(st, self.last_error())
        if out is not None and out.dtype == MEETING_DTYPE and out.flags.c_contiguous and out.shape[0] >= n.value:
            if n.value:
                st = self.lib.glint_meetings(self.h, out.ctypes.data_as(ctypes.c_void_p), n.value, ctypes.byref(n))
                if st != 0:
                    raise GlintError(st, self.last_error())
            return out[: n.value]
        out = np.zeros(n.value, dtype=MEETING_DTYPE)
        if n.value:
            st = self.lib.glint_meetings(self.h, out.ctypes.data_as(ctypes.c_void_p), n.value, ctypes.byref(n))
            if st != 0:
                raise GlintError(st, self.last_error())
        return out

    def active_search(self, pids, cap: int | None = None) -> np.ndarray:
        """Active meetings of the listed objects after the last step
        (search_multi, cuda/geometry.cu:605-663), in bucket order."""
        p = np.ascontiguousarray(pids, dtype=np.uint32)
        n = ctypes.c_uint64()
        if cap is None:
            st = self.lib.glint_active_search(self.h, p.ctypes.data_as(ctypes.c_void_p), p.shape[0], None, 0,
                                              ctypes.byref(n))
            if st != 0:
                raise GlintError(st, self.last_error())
            cap = n.value
        out = np.zeros(int(cap), dtype=SEARCH_DTYPE)
        st = self.lib.glint_active_search(self.h, p.ctypes.data_as(ctypes.c_void_p), p.shape[0],
                                          out.ctypes.data_as(ctypes.c_void_p) if cap else None, int(cap),
                                          ctypes.byref(n))
        if st != 0:
            raise GlintError(st, self.last_error())
        return out[: min(int(n.value), int(cap))]

    def precision_probe(self, stride: int = 256) -> dict:
        """The FP32 screen of the precision form against the reference's FP64
        distance test on pairs sampled from the last step (every stride-th
        object of the leaf-major order with its 32 successors)."""
        rep = _abi.GlintPrecisionReport()
        st = self.lib.glint_precision_probe(self.h, int(stride), ctypes.byref(rep))
        if st != 0:
            raise GlintError(st, self.last_error())
        return rep.as_dict()

    # -- key-value store -----------------------------------------------------
    def flush(self) -> "_abi.GlintStoreInfo":
        """Flush the pending keys into the store now (cuda/geometry.cu:1752-2135)."""
        info = _abi.GlintStoreInfo()
        st = self.lib.glint_flush(self.h, ctypes.byref(info))
        if st != 0:
            raise GlintError(st, self.last_error())
        return info

    def serve_only(self, reserve: int = 8 << 30) -> int:
        """Keep only what queries need (glint_serve_only): the step state is
        released and host-kept blocks move onto the device while `reserve`
        bytes stay free; returns the blocks on the device."""
        n = ctypes.c_uint32()
        st = self.lib.glint_serve_only(self.h, int(reserve), ctypes.byref(n))
        if st != 0:
            raise GlintError(st, self.last_error())
        return int(n.value)

    def store(self) -> dict:
        """The last flush's store as host arrays (the reference's h_keys,
        h_sids, h_CTF_capacity, h_ctfs, h_bitmaps and oversize buffer)."""
        info = _abi.GlintStoreInfo()
        st = self.lib.glint_store_read(self.h, None, None, None, None, None, None, None, None, ctypes.byref(info))
        if st != 0:
            raise GlintError(st, self.last_error())
        C = self.config.CTF_count or 100
        out = {"keys": np.zeros(int(info.key_bytes), np.uint8), "sids": np.zeros(self.n, np.uint16),
               "ctf_capacity": np.zeros(C, np.uint32), "ctfs": np.zeros(C, _abi.CTF_META_DTYPE),
               "bitmaps": np.zeros(C * _abi.BITMAP_BYTES, np.uint8),
               "o_keys": np.zeros((int(info.oversize_kv_count), 16), np.uint8),
               "o_boxes": np.zeros((int(info.oversize_kv_count), 4), np.float32),
               "o_bitmap": np.zeros(_abi.BITMAP_BYTES, np.uint8)}
        ptr = lambda a: a.ctypes.data_as(ctypes.c_void_p)  # noqa: E731
        st = self.lib.glint_store_read(self.h, ptr(out["keys"]), ptr(out["sids"]), ptr(out["ctf_capacity"]),
                                       ptr(out["ctfs"]), ptr(out["bitmaps"]), ptr(out["o_keys"]),
                                       ptr(out["o_boxes"]), ptr(out["o_bitmap"]), ctypes.byref(info))
        if st != 0:
            raise GlintError(st, self.last_error())
        out["info"] = info
        return out

    def dump_store(self, raid_path: str, meta_path: str, prefix: str, ctb: int = 0):
        """The last flush's store into files in the reference's layout
        (straight_dump, tracing/process.cpp:254-348)."""
        st = self.lib.glint_store_dump(self.h, raid_path.encode(), meta_path.encode(), prefix.encode(), int(ctb))
        if st != 0:
            raise GlintError(st, self.last_error())

    def load_store(self, raid_path: str, meta_path: str, prefix: str, ctb: int = 0, ctf_count: int | None = None):
        """One block's files (written here or by the reference) into a kept
        block for queries (workbench::load_CTB_meta and friends); ctf_count
        for a compacted block (its record does not carry it)."""
        if ctf_count is None:
            st = self.lib.glint_store_load(self.h, raid_path.encode(), meta_path.encode(), prefix.encode(), int(ctb))
        else:
            st = self.lib.glint_store_load_ctfs(self.h, raid_path.encode(), meta_path.encode(), prefix.encode(),
                                                int(ctb), int(ctf_count))
        if st != 0:
            raise GlintError(st, self.last_error())

    def store_blocks(self) -> int:
        return int(self.lib.glint_store_blocks(self.h))

    def block_info(self, block: int) -> "_abi.GlintBlockInfo":
        info = _abi.GlintBlockInfo()
        st = self.lib.glint_store_block_info(self.h, int(block), ctypes.byref(info))
        if st != 0:
            raise GlintError(st, self.last_error())
        return info

    def block(self, block: int) -> dict:
        """A kept block (0 = the oldest) as host arrays, in the layout of
        store(); "times" are the CTB record's, "o_times" the oversize
        buffer's."""
        bi = self.block_info(block)
        info = bi.store
        C = int(bi.CTF_count)
        out = {"keys": np.zeros(int(info.key_bytes), np.uint8), "sids": np.zeros(self.n, np.uint16),
               "ctfs": np.zeros(C, _abi.CTF_META_DTYPE), "bitmaps": np.zeros(C * _abi.BITMAP_BYTES, np.uint8),
               "o_keys": np.zeros((int(info.oversize_kv_count), 16), np.uint8),
               "o_boxes": np.zeros((int(info.oversize_kv_count), 4), np.float32),
               "o_bitmap": np.zeros(_abi.BITMAP_BYTES, np.uint8)}
        ptr = lambda a: a.ctypes.data_as(ctypes.c_void_p)  # noqa: E731
        st = self.lib.glint_store_block_read(self.h, int(block), ptr(out["keys"]), ptr(out["sids"]),
                                             ptr(out["ctfs"]), ptr(out["bitmaps"]), ptr(out["o_keys"]),
                                             ptr(out["o_boxes"]), ptr(out["o_bitmap"]))
        if st != 0:
            raise GlintError(st, self.last_error())
        out["ctf_capacity"] = out["ctfs"]["CTF_kv_capacity"].copy()
        out["times"] = list(bi.times)
        out["o_times"] = [info.oversize_start_time_min, info.oversize_start_time_max, info.oversize_end_time_min,
                          info.oversize_end_time_max]
        out["info"] = info
        return out

    def dump_block(self, block: int, raid_path: str, meta_path: str, prefix: str, ctb: int = 0):
        """A kept block into files in the reference's layout."""
        st = self.lib.glint_store_block_dump(self.h, int(block), raid_path.encode(), meta_path.encode(),
                                             prefix.encode(), int(ctb))
        if st != 0:
            raise GlintError(st, self.last_error())

    def compact(self, first: int, count: int, split_num: int) -> dict:
        """Merge kept blocks [first, first + count) into one block of
        split_num^2 CTFs (merge_dump, tools/compaction.cpp:729-1215), which
        takes their place among the kept blocks."""
        info = _abi.GlintCompactInfo()
        st = self.lib.glint_store_compact(self.h, int(first), int(count), int(split_num), ctypes.byref(info))
        if st != 0:
            raise GlintError(st, self.last_error())
        return info.as_dict()

    def query(self, queries):
        """Contact-trace queries over the kept store blocks.  queries: a list of
        (seeds, hops, t_start, t_end); returns, per query, a list of per-hop
        arrays of newly reached object ids (ascending), and the keys scanned."""
        n = len(queries)
        qs = (_abi.GlintQuery * max(n, 1))()
        rs = (_abi.GlintQueryResult * max(n, 1))()
        keep = []
        for i, (seeds, hops, t0, t1) in enumerate(queries):
            sd = np.ascontiguousarray(seeds, dtype=np.uint32)
            keep.append(sd)
            qs[i].seeds = sd.ctypes.data_as(ctypes.c_void_p).value if sd.size else None
            qs[i].n_seeds, qs[i].hops, qs[i].t_start, qs[i].t_end = sd.size, int(hops), int(t0), int(t1)
            rs[i].ids, rs[i].cap = None, 0
        st = self.lib.glint_query_batch(self.h, qs, n, rs)
        if st != 0:
            raise GlintError(st, self.last_error())
        bufs = []
        for i in range(n):
            b = np.zeros(max(int(rs[i].n), 1), np.uint32)
            bufs.append(b)
            rs[i].ids, rs[i].cap = b.ctypes.data_as(ctypes.c_void_p).value, b.size
        st = self.lib.glint_query_batch(self.h, qs, n, rs)
        if st != 0:
            raise GlintError(st, self.last_error())
        out = []
        for i, (seeds, hops, t0, t1) in enumerate(queries):
            ends = [0] + [int(rs[i].hop_end[h]) for h in range(int(hops))]
            out.append([bufs[i][ends[h]:ends[h + 1]] for h in range(int(hops))])
        return out, sum(int(rs[i].keys_scanned) for i in range(n))

    # -- state ------------------------------------------------------------------
    def schema(self):
        nodes = np.zeros(self.schema_capacity, dtype=SCHEMA_DTYPE)
        ss = np.zeros(self.schema_capacity, dtype=np.uint32)
        gs = np.zeros(self.grids_capacity, dtype=np.uint32)
        gc = np.zeros(self.grids_capacity, dtype=np.uint32)
        ssi = ctypes.c_uint32()
        gsi = ctypes.c_uint32()
        st = self.lib.glint_get_schema(self.h, nodes.ctypes.data_as(ctypes.c_void_p), ss.ctypes.data_as(ctypes.c_void_p),
                                       gs.ctypes.data_as(ctypes.c_void_p), gc.ctypes.data_as(ctypes.c_void_p),
                                       ctypes.byref(ssi), ctypes.byref(gsi))
        if st != 0:
            raise GlintError(st, self.last_error())
        return nodes, ss, gs, gc, ssi.value, gsi.value

    def buckets(self):
        B = int(self.num_buckets)
        k = np.zeros(B, np.uint64)
        s = np.zeros(B, np.uint32)
        m = np.zeros((B, 4), np.float32)
        st = self.lib.glint_get_buckets(self.h, k.ctypes.data_as(ctypes.c_void_p), s.ctypes.data_as(ctypes.c_void_p),
                                        m.ctypes.data_as(ctypes.c_void_p))
        if st != 0:
            raise GlintError(st, self.last_error())
        return k, s, m

    @property
    def stream(self) -> int:
        return int(self.lib.glint_stream(self.h) or 0)

    def last_error(self) -> str:
        return self.lib.glint_last_error(self.h).decode()

    def snapshot(self, path: str):
        """Everything the next steps read, into one file (glint_snapshot_save)."""
        st = self.lib.glint_snapshot_save(self.h, path.encode())
        if st != 0:
            raise GlintError(st, self.last_error())

    @classmethod
    def resume(cls, path: str, config: Configuration, device: int = -1) -> "DeviceBench":
        """A context that continues from a snapshot (glint_snapshot_load);
        `config` is the configuration the snapshot was taken with."""
        lib = _abi.lib()
        h = ctypes.c_void_p()
        st = lib.glint_snapshot_load(path.encode(), int(device), ctypes.byref(h))
        if st != 0:
            raise GlintError(st, "glint_snapshot_load")
        b = cls._view(h.value, config)
        b._owned = True
        return b

    @classmethod
    def _view(cls, handle: int, config: Configuration):
        """A DeviceBench over a context owned elsewhere (a batch region)."""
        b = cls.__new__(cls)
        b.lib = _abi.lib()
        b.config = config
        b.n = int(config.num_objects)
        b.h = ctypes.c_void_p(handle)
        b._owned = False
        sc, gc, bk = ctypes.c_uint32(), ctypes.c_uint32(), ctypes.c_uint64()
        b.lib.glint_get_capacities(b.h, ctypes.byref(sc), ctypes.byref(gc), ctypes.byref(bk))
        b.schema_capacity, b.grids_capacity, b.num_buckets = sc.value, gc.value, bk.value
        return b

    def close(self):
        if getattr(self, "h", None):
            if getattr(self, "_owned", True):
                self.lib.glint_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class TraceFiles:
    """The reference's trace chunk files (<prefix><st>_<N>.tr, 100 steps
    each), read ahead on a host thread into page-locked step buffers
    (glint_trace_*).  step(t) returns an (N, 2) view valid until two more
    steps have been asked for."""

    def __init__(self, prefix: str, num_objects: int, first_step: int, num_steps: int, ring: int = 4):
        self.lib = _abi.lib()
        self.n = int(num_objects)
        h = ctypes.c_void_p()
        st = self.lib.glint_trace_open(prefix.encode(), self.n, int(first_step), int(num_steps), int(ring),
                                       ctypes.byref(h))
        if st != 0:
            raise GlintError(st, self.lib.glint_trace_error().decode())
        self.h = h

    def step(self, t: int) -> np.ndarray:
        ptr = ctypes.c_void_p()
        st = self.lib.glint_trace_step(self.h, int(t), ctypes.byref(ptr))
        if st != 0:
            raise GlintError(st, self.lib.glint_trace_error().decode())
        raw = (ctypes.c_double * (2 * self.n)).from_address(ptr.value)
        return np.frombuffer(raw, dtype=np.float64).reshape(self.n, 2)

    def close(self):
        if getattr(self, "h", None):
            self.lib.glint_trace_close(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def write_trace_files(prefix: str, first_step: int, points: np.ndarray):
    """steps of points (steps, N, 2) into the reference's chunk files"""
    p = np.ascontiguousarray(points, dtype=np.float64)
    lib = _abi.lib()
    st = lib.glint_trace_write(prefix.encode(), int(p.shape[1]), int(first_step), p.ctypes.data, int(p.shape[0]))
    if st != 0:
        raise GlintError(st, lib.glint_trace_error().decode())


class Pipe:
    """Pipelined stepping from page-locked host memory (glint_pipe_*): the
    next step's points are copied while the current step computes, and each
    step's meetings land in page-locked result buffers.  submit(points, t)
    finishes the step before; result(t) gives (stats, meetings) of the last
    finished step, a view valid until the submit two steps later."""

    def __init__(self, bench: DeviceBench, result_capacity: int = 0):
        self.lib = bench.lib
        self.bench = bench
        h = ctypes.c_void_p()
        st = self.lib.glint_pipe_create(bench.h, int(result_capacity), ctypes.byref(h))
        if st != 0:
            raise GlintError(st, bench.last_error())
        self.h = h
        self._keep = [None, None]

    def submit(self, points, cur_time: int):
        """points: an (N, 2) float64 array, ideally from pinned_empty (other
        memory is copied synchronously by the driver)."""
        p = np.ascontiguousarray(points, dtype=np.float64)
        st = self.lib.glint_pipe_submit(self.h, p.ctypes.data_as(ctypes.c_void_p), int(cur_time))
        if st != 0:
            raise GlintError(st, self.bench.last_error())
        self._keep = [self._keep[1], p]

    def result(self, cur_time: int):
        stats = GlintStepStats()
        ptr = ctypes.c_void_p()
        n = ctypes.c_uint64()
        st = self.lib.glint_pipe_result(self.h, int(cur_time), ctypes.byref(stats), ctypes.byref(ptr),
                                        ctypes.byref(n))
        if st != 0:
            raise GlintError(st, self.bench.last_error())
        if n.value == 0:
            return stats, np.zeros(0, MEETING_DTYPE)
        raw = (ctypes.c_uint8 * (MEETING_DTYPE.itemsize * n.value)).from_address(ptr.value)
        return stats, np.frombuffer(raw, dtype=MEETING_DTYPE)

    def close(self):
        if getattr(self, "h", None):
            self.lib.glint_pipe_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Server:
    """Continuous-batching query server over a DeviceBench's kept store blocks
    (glint_server_*)."""

    def __init__(self, bench: DeviceBench, max_slots: int = 64):
        self.bench = bench
        self.lib = bench.lib
        h = ctypes.c_void_p()
        st = self.lib.glint_server_create(bench.h, int(max_slots), ctypes.byref(h))
        if st != 0:
            raise GlintError(st, bench.last_error())
        self.h = h
        self.slots = int(self.lib.glint_server_slots(h))
        self._keep = {}

    def submit(self, seeds, hops: int, t_start: int = 0, t_end: int = 0) -> int:
        sd = np.ascontiguousarray(seeds, dtype=np.uint32)
        q = _abi.GlintQuery()
        q.seeds = sd.ctypes.data_as(ctypes.c_void_p).value if sd.size else None
        q.n_seeds, q.hops, q.t_start, q.t_end = sd.size, int(hops), int(t_start), int(t_end)
        t = ctypes.c_uint64()
        st = self.lib.glint_server_submit(self.h, ctypes.byref(q), ctypes.byref(t))
        if st != 0:
            raise GlintError(st, self.bench.last_error())
        self._keep[t.value] = int(hops)
        return t.value

    def step(self):
        a, q = ctypes.c_uint32(), ctypes.c_uint32()
        st = self.lib.glint_server_step(self.h, ctypes.byref(a), ctypes.byref(q))
        if st != 0:
            raise GlintError(st, self.bench.last_error())
        return a.value, q.value

    def poll(self, ticket: int, cap: int = 1 << 20):
        """None while running; else (per-hop id arrays, keys scanned)"""
        buf = np.zeros(max(cap, 1), np.uint32)
        r = _abi.GlintQueryResult()
        r.ids, r.cap = buf.ctypes.data_as(ctypes.c_void_p).value, buf.size
        done = ctypes.c_int()
        st = self.lib.glint_server_poll(self.h, int(ticket), ctypes.byref(r), ctypes.byref(done))
        if st != 0:
            raise GlintError(st, self.bench.last_error())
        if not done.value:
            return None
        hops = self._keep.pop(int(ticket))
        ends = [0] + [min(int(r.hop_end[h]), buf.size) for h in range(hops)]
        return [buf[ends[h]:ends[h + 1]] for h in range(hops)], int(r.keys_scanned), int(r.n)

    def close(self):
        if getattr(self, "h", None):
            self.lib.glint_server_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def write_store_files(store: dict, info, num_objects: int, raid_path: str, meta_path: str, prefix: str,
                      ctb: int = 0):
    """Host store arrays (as DeviceBench.store() returns them; `info` a
    glint_store_info-layout structure) into files in the reference's layout,
    without a device (glint_store_write)."""
    lib = _abi.lib()
    C = int(store["ctfs"].shape[0])
    arrs = {k: np.ascontiguousarray(store[k]) for k in ("keys", "sids", "ctfs", "bitmaps", "o_keys", "o_boxes",
                                                        "o_bitmap")}
    v = _abi.GlintStoreView()
    v.num_objects, v.CTF_count = int(num_objects), C
    ptr = lambda a: a.ctypes.data if a.size else None  # noqa: E731
    v.keys, v.sids, v.ctfs, v.bitmaps = ptr(arrs["keys"]), ptr(arrs["sids"]), ptr(arrs["ctfs"]), ptr(arrs["bitmaps"])
    v.oversize_keys, v.oversize_boxes, v.oversize_bitmap = ptr(arrs["o_keys"]), ptr(arrs["o_boxes"]), \
        ptr(arrs["o_bitmap"])
    ctypes.memmove(ctypes.addressof(v.info), ctypes.addressof(info), ctypes.sizeof(v.info))
    st = lib.glint_store_write(ctypes.byref(v), raid_path.encode(), meta_path.encode(), prefix.encode(), int(ctb))
    if st != 0:
        raise GlintError(st, lib.glint_store_file_error().decode())


def pinned_empty(shape, dtype) -> np.ndarray:
    """An uninitialised array in page-locked host memory (glint_host_alloc),
    released when the array and its views are gone."""
    import weakref
    dt = np.dtype(dtype)
    count = int(np.prod(shape))
    nbytes = max(count * dt.itemsize, 1)
    lib = _abi.lib()
    p = ctypes.c_void_p()
    st = lib.glint_host_alloc(nbytes, ctypes.byref(p))
    if st != 0 or not p.value:
        raise GlintError(st, "glint_host_alloc")
    raw = (ctypes.c_uint8 * nbytes).from_address(p.value)
    arr = np.frombuffer(raw, dtype=np.uint8, count=count * dt.itemsize).view(dt).reshape(shape)
    weakref.finalize(raw, lib.glint_host_free, ctypes.c_void_p(p.value))
    return arr


def cuda_create_device_bench(config: Configuration, mbr, first_points=None, schema=None) -> DeviceBench:
    """Mirror of cuda_create_device_bench (cuda/geometry.cu:1395-1565)."""
    return DeviceBench(config, mbr, first_points, schema)


def process_with_gpu(bench: DeviceBench, points, cur_time: int) -> GlintStepStats:
    """Mirror of process_with_gpu (cuda/geometry.cu:1573-2218) for one timestep."""
    return bench.step(points, cur_time)
