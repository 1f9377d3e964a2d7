"""Seeded synthetic Manhattan-grid trajectories (host side).

Stand-in for the reference's trace chunks (timestep-major ``Point[N*100]``
arrays of FP64 lon/lat, tracing/process.cpp:128-144).  The C implementation
lives in csrc/tracegen.h and is shared bit-for-bit with the device generator.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB = None

# seeds of the benchmark workloads: 0x474C494E54 is "GLINT"
SEED_SMALL = 0x474C494E54000000
SEED_SCALE = 0x474C494E54000001
SEED_SKEW = 0x474C494E54000002
SEED_REGIONS = 0x474C494E54000003
SEED_SERVING = 0x474C494E54000004
SEED_QUERIES = 0x474C494E54000005


def _lib():
    global _LIB
    if _LIB is None:
        path = os.path.join(_HERE, "_tracegen.so")
        if not os.path.exists(path):
            from . import build as _build
            _build.build_tracegen()
        lib = ctypes.CDLL(path)
        lib.tg_create.restype = ctypes.c_void_p
        lib.tg_create.argtypes = [ctypes.c_uint64, ctypes.c_uint32, ctypes.c_int]
        lib.tg_set_shape.argtypes = [ctypes.c_void_p, ctypes.c_double, ctypes.c_double, ctypes.c_uint32,
                                     ctypes.c_double, ctypes.c_double, ctypes.c_double]
        lib.tg_generate.argtypes = [ctypes.c_void_p, ctypes.c_uint32, ctypes.c_void_p]
        lib.tg_box.argtypes = [ctypes.c_void_p, ctypes.c_void_p]
        lib.tg_get_params.restype = ctypes.c_void_p
        lib.tg_get_params.argtypes = [ctypes.c_void_p]
        lib.tg_params_size.restype = ctypes.c_uint32
        lib.tg_object_size.restype = ctypes.c_uint32
        lib.tg_get_objects.argtypes = [ctypes.c_void_p, ctypes.c_void_p]
        lib.tg_current_step.restype = ctypes.c_uint32
        lib.tg_current_step.argtypes = [ctypes.c_void_p]
        lib.tg_destroy.argtypes = [ctypes.c_void_p]
        _LIB = lib
    return _LIB


class TraceGenerator:
    """Produces consecutive 1-second steps of N objects as (N, 2) float64 arrays.

    kind 0: 40x40 km box, 100 m blocks, 8 hotspots (sigma 500 m) holding 70% of
    the objects, 30% uniform, 10% stationary, speeds U(0.5, 2) m/s.
    kind 1: extreme skew, 5 hotspots with sigma 50 m holding 20%, the rest uniform.
    """

    def __init__(self, seed: int, num_objects: int, kind: int = 0, *, extent_m: float | None = None,
                 block_m: float = 100.0, n_hotspots: int | None = None, sigma_m: float | None = None,
                 hotspot_frac: float | None = None, stationary_frac: float = 0.1):
        self.lib = _lib()
        self.n = int(num_objects)
        self.h = self.lib.tg_create(ctypes.c_uint64(seed), self.n, int(kind))
        if not self.h:
            raise MemoryError("tg_create failed")
        if any(v is not None for v in (extent_m, n_hotspots, sigma_m, hotspot_frac)) or stationary_frac != 0.1:
            d_ext = 40000.0 if extent_m is None else float(extent_m)
            d_nh = (8 if kind == 0 else 5) if n_hotspots is None else int(n_hotspots)
            d_sig = (500.0 if kind == 0 else 50.0) if sigma_m is None else float(sigma_m)
            d_hf = (0.7 if kind == 0 else 0.2) if hotspot_frac is None else float(hotspot_frac)
            self.lib.tg_set_shape(self.h, d_ext, float(block_m), d_nh, d_sig, d_hf, float(stationary_frac))

    def box(self) -> np.ndarray:
        out = np.zeros(4, dtype=np.float64)
        self.lib.tg_box(self.h, out.ctypes.data)
        return out

    def steps(self, nsteps: int) -> np.ndarray:
        out = np.empty((nsteps, self.n, 2), dtype=np.float64)
        self.lib.tg_generate(self.h, nsteps, out.ctypes.data)
        return out

    def params_bytes(self) -> bytes:
        size = self.lib.tg_params_size()
        return ctypes.string_at(self.lib.tg_get_params(self.h), size)

    def objects_bytes(self) -> bytes:
        buf = ctypes.create_string_buffer(self.lib.tg_object_size() * max(self.n, 1))
        self.lib.tg_get_objects(self.h, buf)
        return buf.raw[: self.lib.tg_object_size() * self.n]

    @property
    def step_index(self) -> int:
        return int(self.lib.tg_current_step(self.h))

    def close(self):
        if self.h:
            self.lib.tg_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
