"""ctypes declarations of the C ABI in include/glint.h."""
from __future__ import annotations

import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
library_path = os.path.join(HERE, "libglint.so")

_LIB = None

STATUS = {
    0: "ok", 1: "invalid argument", 2: "CUDA error", 3: "out of device memory",
    4: "device buffer capacity exceeded", 5: "unsupported configuration", 6: "invalid context state",
    7: "no CUDA device",
}


class GlintError(RuntimeError):
    def __init__(self, status: int, detail: str = ""):
        self.status = int(status)
        super().__init__(f"glint status {status} ({STATUS.get(int(status), '?')}): {detail}")


class GlintConfig(ctypes.Structure):
    _fields_ = [
        ("num_objects", ctypes.c_uint32),
        ("grid_capacity", ctypes.c_uint32),
        ("grid_amplify", ctypes.c_double),
        ("num_meeting_buckets", ctypes.c_uint64),
        ("reach_distance", ctypes.c_double),
        ("min_meet_time", ctypes.c_uint32),
        ("max_meet_time", ctypes.c_uint32),
        ("schema_update_delay", ctypes.c_uint32),
        ("dynamic_schema", ctypes.c_uint32),
        ("phased_lookup", ctypes.c_uint32),
        ("start_time", ctypes.c_uint32),
        ("x_buffer", ctypes.c_double),
        ("y_buffer", ctypes.c_double),
        ("G_bytes", ctypes.c_uint32),
        ("CTF_count", ctypes.c_uint32),
        ("dProbFalse", ctypes.c_double),
        ("precision_mode", ctypes.c_uint32),
        ("device", ctypes.c_uint32),
        ("new_capacity", ctypes.c_uint64),
        ("check_capacity", ctypes.c_uint64),
        ("meeting_log_capacity", ctypes.c_uint64),
        ("timing", ctypes.c_uint32),
        ("auto_flush", ctypes.c_uint32),
        ("split_num", ctypes.c_uint32),
        ("store_keep", ctypes.c_uint32),
        ("kv_restriction", ctypes.c_uint64),
        ("kv_capacity", ctypes.c_uint64),
        ("use_graph", ctypes.c_uint32),
        ("store_host_keep", ctypes.c_uint32),
        ("refine_chunk", ctypes.c_uint32),
        ("reserved3", ctypes.c_uint32),
    ]


class GlintBox(ctypes.Structure):
    _fields_ = [("low", ctypes.c_double * 2), ("high", ctypes.c_double * 2)]


class GlintSchemaInit(ctypes.Structure):
    _fields_ = [
        ("nodes", ctypes.c_void_p),
        ("num_nodes", ctypes.c_uint32),
        ("schema_stack_index", ctypes.c_uint32),
        ("grids_stack_index", ctypes.c_uint32),
        ("reserved", ctypes.c_uint32),
        ("schema_stack", ctypes.c_void_p),
        ("grids_stack", ctypes.c_void_p),
    ]


class GlintStepStats(ctypes.Structure):
    _fields_ = [
        ("cur_time", ctypes.c_uint32),
        ("checks", ctypes.c_uint32),
        ("border_objects", ctypes.c_uint32),
        ("cross_checks", ctypes.c_uint32),
        ("candidates", ctypes.c_uint64),
        ("contacts", ctypes.c_uint64),
        ("new_keys", ctypes.c_uint64),
        ("num_taken_buckets", ctypes.c_uint64),
        ("num_active_meetings", ctypes.c_uint32),
        ("meetings", ctypes.c_uint32),
        ("splits", ctypes.c_uint32),
        ("merges", ctypes.c_uint32),
        ("leaves", ctypes.c_uint32),
        ("nodes", ctypes.c_uint32),
        ("dropped_objects", ctypes.c_uint32),
        ("rechecks", ctypes.c_uint32),
        ("ambiguous", ctypes.c_uint32),
        ("band_pairs", ctypes.c_uint32),
        ("error_flags", ctypes.c_uint32),
        ("launches", ctypes.c_uint32),
        ("meeting_log_size", ctypes.c_uint64),
        ("ms", ctypes.c_float * 8),
        ("kv_count", ctypes.c_uint64),
        ("flushed", ctypes.c_uint32),
        ("flush_ms", ctypes.c_float),
        ("box_band", ctypes.c_uint32),
        ("reserved1", ctypes.c_uint32),
    ]

    def as_dict(self):
        d = {f: getattr(self, f) for f, _ in self._fields_ if f != "ms"}
        d["ms"] = list(self.ms)
        return d


MEETING_DTYPE = np.dtype([("pid1", "<u4"), ("pid2", "<u4"), ("start", "<u4"), ("end", "<u4"), ("mbr", "<f4", (4,))])
SCHEMA_DTYPE = np.dtype([
    ("grid_id", "<u4"), ("level", "<i2"), ("type", "<i2"), ("overflow_count", "<i2"),
    ("underflow_count", "<i2"), ("pad", "<u4"), ("mid_x", "<f8"), ("mid_y", "<f8"),
    ("low", "<f8", (2,)), ("high", "<f8", (2,)), ("children", "<u4", (4,)),
])
assert SCHEMA_DTYPE.itemsize == 80 and MEETING_DTYPE.itemsize == 32
# glint_ctf_meta: CTF (tracing/step_merge.h) without its pointers
CTF_META_DTYPE = np.dtype([("ctf_mbr", "<f4", (4,)), ("CTF_kv_capacity", "<u4"), ("start_time_min", "<u4"),
                           ("start_time_max", "<u4"), ("end_time_min", "<u4"), ("end_time_max", "<u4"),
                           ("ctf_bitmap_size", "<u4"), ("key_bit", "<u2"), ("id_bit", "<u2"),
                           ("duration_bit", "<u2"), ("end_bit", "<u2"), ("low_x_bit", "<u2"), ("low_y_bit", "<u2"),
                           ("edge_bit", "<u2"), ("mbr_bit", "<u2"), ("x_grid", "<u2"), ("y_grid", "<u2"),
                           ("reserved", "<u4")])
assert CTF_META_DTYPE.itemsize == 64
BITMAP_BYTES = 256 * 256 // 8


class GlintStoreInfo(ctypes.Structure):
    _fields_ = [("kv_count", ctypes.c_uint64), ("key_bytes", ctypes.c_uint64), ("oversize_kv_count", ctypes.c_uint32),
                ("oversize_start_time_min", ctypes.c_uint32), ("oversize_start_time_max", ctypes.c_uint32),
                ("oversize_end_time_min", ctypes.c_uint32), ("oversize_end_time_max", ctypes.c_uint32),
                ("sid_count", ctypes.c_uint32), ("oversize_oid_count", ctypes.c_uint32),
                ("end_time_min", ctypes.c_uint32), ("cur_time", ctypes.c_uint32), ("reserved", ctypes.c_uint32),
                ("bits_outside", ctypes.c_uint64)]

    def as_dict(self):
        return {f: getattr(self, f) for f, _ in self._fields_ if f != "reserved"}


class GlintStoreView(ctypes.Structure):
    _fields_ = [("num_objects", ctypes.c_uint32), ("CTF_count", ctypes.c_uint32), ("keys", ctypes.c_void_p),
                ("sids", ctypes.c_void_p), ("ctfs", ctypes.c_void_p), ("bitmaps", ctypes.c_void_p),
                ("oversize_keys", ctypes.c_void_p), ("oversize_boxes", ctypes.c_void_p),
                ("oversize_bitmap", ctypes.c_void_p), ("info", GlintStoreInfo)]


class GlintBlockInfo(ctypes.Structure):
    """glint_block_info: a kept block's CTF count, CTB record times and sizes"""
    _fields_ = [("CTF_count", ctypes.c_uint32), ("times", ctypes.c_uint32 * 4), ("reserved", ctypes.c_uint32),
                ("store", GlintStoreInfo)]


class GlintCompactInfo(ctypes.Structure):
    _fields_ = [("CTF_count", ctypes.c_uint32), ("blocks", ctypes.c_uint32), ("kv_count", ctypes.c_uint64),
                ("key_bytes", ctypes.c_uint64), ("padding", ctypes.c_uint64), ("oversize_kv_count", ctypes.c_uint32),
                ("sid_count", ctypes.c_uint32), ("x_part", ctypes.c_uint32), ("y_part", ctypes.c_uint32),
                ("ms", ctypes.c_float), ("reserved", ctypes.c_uint32)]

    def as_dict(self):
        return {f: getattr(self, f) for f, _ in self._fields_ if f != "reserved"}


class GlintQuery(ctypes.Structure):
    _fields_ = [("seeds", ctypes.c_void_p), ("n_seeds", ctypes.c_uint32), ("hops", ctypes.c_uint32),
                ("t_start", ctypes.c_uint32), ("t_end", ctypes.c_uint32)]


class GlintQueryResult(ctypes.Structure):
    _fields_ = [("ids", ctypes.c_void_p), ("cap", ctypes.c_uint64), ("n", ctypes.c_uint64),
                ("hop_end", ctypes.c_uint64 * 8), ("keys_scanned", ctypes.c_uint64)]


class GlintPrecisionReport(ctypes.Structure):
    _fields_ = [("pairs", ctypes.c_uint64), ("in_band", ctypes.c_uint64), ("mismatches", ctypes.c_uint64),
                ("contacts", ctypes.c_uint64), ("max_abs_err_m", ctypes.c_double),
                ("max_abs_err_near_m", ctypes.c_double), ("max_band_m", ctypes.c_double),
                ("stride", ctypes.c_uint32), ("reserved", ctypes.c_uint32)]

    def as_dict(self):
        return {f: getattr(self, f) for f, _ in self._fields_ if f != "reserved"}


# glint_search_info = search_info_unit (tracing/workbench.h:85-88)
SEARCH_DTYPE = np.dtype([("pid", "<u4"), ("target", "<u4"), ("start", "<u4"), ("end", "<u4"), ("mbr", "<f4", (4,))])
assert SEARCH_DTYPE.itemsize == 32


def load_library(path: str | None = None):
    """Loads libglint.so; builds it in-tree first when it is missing."""
    p = path or library_path
    if not os.path.exists(p):
        from . import build as _build
        _build.build()
    lib = ctypes.CDLL(p)
    vp = ctypes.c_void_p
    u32, u64 = ctypes.c_uint32, ctypes.c_uint64
    lib.glint_abi_version.restype = ctypes.c_int
    lib.glint_struct_sizes.argtypes = [ctypes.POINTER(ctypes.c_uint32)]
    lib.glint_status_string.restype = ctypes.c_char_p
    lib.glint_status_string.argtypes = [ctypes.c_int]
    lib.glint_config_defaults.argtypes = [ctypes.POINTER(GlintConfig), u32]
    lib.glint_create.argtypes = [ctypes.POINTER(GlintConfig), ctypes.POINTER(GlintBox), vp, vp, ctypes.POINTER(vp)]
    lib.glint_destroy.argtypes = [vp]
    lib.glint_last_error.restype = ctypes.c_char_p
    lib.glint_last_error.argtypes = [vp]
    lib.glint_step.argtypes = [vp, vp, u32, ctypes.POINTER(GlintStepStats)]
    lib.glint_step_device.argtypes = [vp, vp, u32]
    lib.glint_sync.argtypes = [vp, ctypes.POINTER(GlintStepStats)]
    lib.glint_meetings.argtypes = [vp, vp, u64, ctypes.POINTER(u64)]
    lib.glint_get_schema.argtypes = [vp, vp, vp, vp, vp, ctypes.POINTER(u32), ctypes.POINTER(u32)]
    lib.glint_get_buckets.argtypes = [vp, vp, vp, vp]
    lib.glint_get_capacities.argtypes = [vp, ctypes.POINTER(u32), ctypes.POINTER(u32), ctypes.POINTER(u64)]
    lib.glint_stream.restype = vp
    lib.glint_stream.argtypes = [vp]
    lib.glint_active_search.argtypes = [vp, vp, u32, vp, u64, ctypes.POINTER(u64)]
    lib.glint_flush.argtypes = [vp, ctypes.POINTER(GlintStoreInfo)]
    lib.glint_serve_only.argtypes = [vp, ctypes.c_uint64, ctypes.POINTER(ctypes.c_uint32)]
    lib.glint_query_batch.argtypes = [vp, ctypes.POINTER(GlintQuery), u32, ctypes.POINTER(GlintQueryResult)]
    lib.glint_store_blocks.restype = u32
    lib.glint_store_blocks.argtypes = [vp]
    lib.glint_server_create.argtypes = [vp, u32, ctypes.POINTER(vp)]
    lib.glint_server_destroy.argtypes = [vp]
    lib.glint_server_slots.restype = u32
    lib.glint_server_slots.argtypes = [vp]
    lib.glint_server_submit.argtypes = [vp, ctypes.POINTER(GlintQuery), ctypes.POINTER(u64)]
    lib.glint_server_step.argtypes = [vp, ctypes.POINTER(u32), ctypes.POINTER(u32)]
    lib.glint_server_poll.argtypes = [vp, u64, ctypes.POINTER(GlintQueryResult), ctypes.POINTER(ctypes.c_int)]
    lib.glint_store_read.argtypes = [vp] * 9 + [ctypes.POINTER(GlintStoreInfo)]
    lib.glint_active_search_noalloc.argtypes = [vp, vp, u32, vp, u64, vp]
    lib.glint_store_write.argtypes = [ctypes.POINTER(GlintStoreView), ctypes.c_char_p, ctypes.c_char_p,
                                      ctypes.c_char_p, u32]
    lib.glint_store_file_error.restype = ctypes.c_char_p
    lib.glint_store_dump.argtypes = [vp, ctypes.c_char_p, ctypes.c_char_p, ctypes.c_char_p, u32]
    lib.glint_store_load.argtypes = [vp, ctypes.c_char_p, ctypes.c_char_p, ctypes.c_char_p, u32]
    lib.glint_store_load_ctfs.argtypes = [vp, ctypes.c_char_p, ctypes.c_char_p, ctypes.c_char_p, u32, u32]
    lib.glint_store_block_info.argtypes = [vp, u32, ctypes.POINTER(GlintBlockInfo)]
    lib.glint_store_block_read.argtypes = [vp, u32] + [vp] * 7
    lib.glint_store_block_dump.argtypes = [vp, u32, ctypes.c_char_p, ctypes.c_char_p, ctypes.c_char_p, u32]
    lib.glint_store_compact.argtypes = [vp, u32, u32, u32, ctypes.POINTER(GlintCompactInfo)]
    lib.glint_snapshot_save.argtypes = [vp, ctypes.c_char_p]
    lib.glint_snapshot_load.argtypes = [ctypes.c_char_p, ctypes.c_int, ctypes.POINTER(vp)]
    lib.glint_trace_open.argtypes = [ctypes.c_char_p, u32, u32, u32, u32, ctypes.POINTER(vp)]
    lib.glint_trace_step.argtypes = [vp, u32, ctypes.POINTER(vp)]
    lib.glint_trace_close.argtypes = [vp]
    lib.glint_trace_error.restype = ctypes.c_char_p
    lib.glint_trace_write.argtypes = [ctypes.c_char_p, u32, u32, vp, u32]
    lib.glint_pipe_create.argtypes = [vp, u64, ctypes.POINTER(vp)]
    lib.glint_pipe_destroy.argtypes = [vp]
    lib.glint_pipe_submit.argtypes = [vp, vp, u32]
    lib.glint_pipe_result.argtypes = [vp, u32, ctypes.POINTER(GlintStepStats), ctypes.POINTER(vp),
                                      ctypes.POINTER(u64)]
    lib.glint_host_alloc.argtypes = [ctypes.c_size_t, ctypes.POINTER(vp)]
    lib.glint_host_free.argtypes = [vp]
    lib.glint_precision_probe.argtypes = [vp, u32, ctypes.POINTER(GlintPrecisionReport)]
    lib.glint_batch_create.argtypes = [u32, vp, vp, vp, ctypes.POINTER(vp)]
    lib.glint_batch_destroy.argtypes = [vp]
    lib.glint_batch_regions.restype = u32
    lib.glint_batch_regions.argtypes = [vp]
    lib.glint_batch_region.restype = vp
    lib.glint_batch_region.argtypes = [vp, u32]
    lib.glint_batch_step.argtypes = [vp, vp, u32]
    lib.glint_batch_sync.argtypes = [vp, vp]
    lib.glint_gen_create.argtypes = [vp, u32, vp, u32, u32, u32, ctypes.POINTER(vp)]
    lib.glint_gen_step.argtypes = [vp, vp, vp]
    lib.glint_gen_destroy.argtypes = [vp]
    return lib


def lib():
    global _LIB
    if _LIB is None:
        _LIB = load_library()
    return _LIB
