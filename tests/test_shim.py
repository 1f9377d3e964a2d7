"""The C++ shim defines the reference's GPU seam with the reference's own
signatures: compiled against the reference headers it exports exactly the
symbols that the reference's process.cpp (built with USE_GPU) leaves
undefined, and it links against libglint.so.  The reference's own GPU-branch
loop and straight_dump then run through the shim on a CPU stand-in for
libglint built from the oracle (oracle/fake_glint.c): the search lists, the
per-step counters and the store files straight_dump writes must equal the
oracle's.  CPU only; skipped where the reference sources are absent."""
import ctypes
import os
import shutil
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
from oracle.bindings import REFERENCE_ROOT as REF  # noqa: E402
SRC = os.path.join(REF, "src")
SHIM = os.path.join(ROOT, "glint_pipeline_gb300", "shim", "glint_ref_shim.cpp")
CUDA_INC = os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "include")

pytestmark = pytest.mark.skipif(not os.path.isdir(os.path.join(SRC, "tracing")) or shutil.which("g++") is None,
                                reason="reference sources or g++ not available")

SEAM = ("_Z24cuda_create_device_benchP9workbenchP8gpu_info", "_Z16process_with_gpuP9workbenchS0_P8gpu_info")


def _flags():
    # the Boost stub stands in for program_options, which util/config.h includes
    return ["-std=c++17", "-O1", "-fPIC", "-w", "-I" + os.path.join(ROOT, "oracle", "ref_stub"), "-I" + SRC,
            "-I" + CUDA_INC, "-I" + os.path.join(ROOT, "include")]


def _symbols(obj):
    out = subprocess.run(["nm", obj], capture_output=True, text=True, check=True).stdout
    syms = {}
    for line in out.splitlines():
        parts = line.split()
        if len(parts) >= 2:
            syms[parts[-1]] = parts[-2]
    return syms


def test_shim_matches_reference_seam(tmp_path):
    shim_o = str(tmp_path / "shim.o")
    proc_o = str(tmp_path / "process.o")
    subprocess.run(["g++", *_flags(), "-c", SHIM, "-o", shim_o], check=True)
    subprocess.run(["g++", *_flags(), "-DUSE_GPU", "-c", os.path.join(SRC, "tracing", "process.cpp"), "-o", proc_o],
                   check=True)
    shim, proc = _symbols(shim_o), _symbols(proc_o)
    for s in SEAM:
        assert proc.get(s) == "U", f"process.cpp does not call {s}"
        assert shim.get(s) == "T", f"shim does not define {s}"


def test_shim_links_against_libglint(tmp_path):
    from glint_pipeline_gb300 import build
    lib = build.build()
    shim_o = str(tmp_path / "shim.o")
    subprocess.run(["g++", *_flags(), "-c", SHIM, "-o", shim_o], check=True)
    so = str(tmp_path / "libshim.so")
    subprocess.run(["g++", "-shared", "-o", so, shim_o, "-L" + os.path.dirname(lib), "-lglint",
                    "-Wl,--no-undefined", "-Wl,--unresolved-symbols=ignore-in-object-files"], check=True)
    undefined = [s for s, k in _symbols(shim_o).items() if k == "U" and s.startswith("glint_")]
    exported = subprocess.run(["nm", "-D", "--defined-only", lib], capture_output=True, text=True).stdout
    for s in undefined:
        assert s in exported, s


class SeamConfig(ctypes.Structure):
    _fields_ = [("num_objects", ctypes.c_uint32), ("grid_capacity", ctypes.c_uint32),
                ("min_meet_time", ctypes.c_uint32), ("max_meet_time", ctypes.c_uint32),
                ("CTF_count", ctypes.c_uint32), ("start_time", ctypes.c_uint32),
                ("num_meeting_buckets", ctypes.c_uint64), ("kv_restriction", ctypes.c_uint64),
                ("reach_distance", ctypes.c_double), ("dProbFalse", ctypes.c_double),
                ("raid_path", ctypes.c_char * 24), ("meta_path", ctypes.c_char * 24)]


def _build_seam(out_dir):
    """the reference's tracing sources (process.cpp with USE_GPU), the shim,
    oracle/ref_seam_driver.cpp and oracle/fake_glint.c in one library"""
    from oracle.bindings import build_oracle
    build_oracle()
    jobs, objs = [], []
    srcs = [(os.path.join(SRC, "tracing", f + ".cpp"), []) for f in
            ("filter", "refinement", "meeting", "workbench", "step_merge", "analyze")]
    srcs += [(os.path.join(SRC, "tracing", "process.cpp"), ["-DUSE_GPU"]), (SHIM, []),
             (os.path.join(ROOT, "oracle", "ref_seam_driver.cpp"), [])]
    for k, (src, extra) in enumerate(srcs):
        o = os.path.join(out_dir, f"s{k}.o")
        jobs.append(subprocess.Popen(["g++", *_flags(), *extra, "-pthread", "-fopenmp", "-c", src, "-o", o]))
        objs.append(o)
    fake = os.path.join(out_dir, "fake.o")
    jobs.append(subprocess.Popen(["gcc", "-O2", "-fPIC", "-std=c11", "-I" + os.path.join(ROOT, "include"),
                                  "-I" + os.path.join(ROOT, "oracle"), "-c",
                                  os.path.join(ROOT, "oracle", "fake_glint.c"), "-o", fake]))
    objs.append(fake)
    assert all(j.wait() == 0 for j in jobs)
    so = os.path.join(out_dir, "libseam.so")
    oracle_dir = os.path.join(ROOT, "oracle")
    subprocess.run(["g++", "-shared", "-o", so, *objs, "-L" + oracle_dir, "-loracle", "-Wl,-rpath," + oracle_dir,
                    "-pthread", "-fopenmp", "-Wl,--no-undefined"], check=True)
    lib = ctypes.CDLL(so)
    vp = ctypes.c_void_p
    lib.seam_create.restype = vp
    lib.seam_create.argtypes = [ctypes.POINTER(SeamConfig), vp, vp]
    lib.seam_step.argtypes = [vp, vp, ctypes.c_uint32]
    lib.seam_search_single.argtypes = [vp, ctypes.c_uint32]
    lib.seam_search_results.restype = ctypes.c_uint32
    lib.seam_search_results.argtypes = [vp, ctypes.c_int, vp, ctypes.c_uint32]
    lib.seam_counts.argtypes = [vp, vp]
    return lib


def test_reference_loop_dumps_the_oracle_store_through_the_shim(tmp_path, monkeypatch):
    """tracer::process's GPU branch through the shim: per-step counters, the
    search_single -> search_multi hand-over, and the flush handed to
    straight_dump, whose files must equal glint_store_write's of the
    oracle's store for the same meetings."""
    from glint_pipeline_gb300 import write_store_files
    from oracle.bindings import SEARCH_DTYPE, Oracle, Store, cantor_inverse, make_config
    from workloads import case_config, make_points
    lib = _build_seam(str(tmp_path))
    monkeypatch.chdir(tmp_path)
    for d in ("r0", "r1", "m", "q0", "q1", "n"):
        os.makedirs(d)
    name, steps, restriction = "dense_20k", 60, 8000
    box, pts = make_points(name, steps)
    cfgd = case_config(name)
    n = cfgd["num_objects"]
    sc = SeamConfig(n, cfgd["grid_capacity"], cfgd["min_meet_time"], 4096, 100, 0, cfgd["num_meeting_buckets"],
                    restriction, cfgd["reach_distance"], 100.0, b"r", b"m")
    o = Oracle(make_config(**cfgd), box, pts[0])
    st = Store(n, box, first_end_time_min=cfgd["min_meet_time"], dProbFalse=100.0, kv_capacity=1 << 22)
    h = lib.seam_create(ctypes.byref(sc), np.ascontiguousarray(box).ctypes.data,
                        np.ascontiguousarray(pts[0]).ctypes.data)
    search_at, targets, flushed_at, dumped_at = 12, None, None, None
    for t in range(steps):
        o.step(pts[t], t)
        mo = o.meetings()
        rec = np.zeros(mo.shape[0], np.dtype([("pid1", "<u4"), ("pid2", "<u4"), ("start", "<u4"),
                                              ("end", "<u4"), ("mbr", "<f4", (4,))]))
        rec["pid1"], rec["pid2"] = cantor_inverse(mo["key"])
        rec["start"], rec["end"], rec["mbr"] = mo["start"], mo["end"], mo["mbr"]
        st.add_meetings(rec)
        if flushed_at is None and st.kv_count > restriction:
            rc, oi = st.flush(t)
            assert rc == 0
            write_store_files(st.result(oi), oi, n, "q", "n", "6oversize_10", 0)
            flushed_at = t
        if t == search_at:
            # an object that is in a meeting long enough to be reported
            busy = o.active_search(np.arange(n, dtype=np.uint32))
            pid = int(busy["pid"][0])
            lib.seam_search_single(h, pid)
        dumped = lib.seam_step(h, np.ascontiguousarray(pts[t]).ctypes.data, t)
        c = o.counts()
        got = np.zeros(6, np.uint64)
        lib.seam_counts(h, got.ctypes.data)
        assert got[:3].tolist() == [c.grid_check_counter, c.num_taken_buckets, c.num_active_meetings], f"step {t}"
        if t == search_at:
            out = np.zeros(1024, SEARCH_DTYPE)
            k = lib.seam_search_results(h, 0, out.ctypes.data, out.shape[0])
            want = o.active_search(np.array([pid], np.uint32))
            assert k == len(want) > 0
            assert out[:k].tobytes() == want.tobytes()
            targets = want["target"].copy()
        if t == search_at + 1:
            out = np.zeros(1 << 16, SEARCH_DTYPE)
            k = lib.seam_search_results(h, 1, out.ctypes.data, out.shape[0])
            want = o.active_search(targets)
            assert k == len(want)
            assert out[:k].tobytes() == want.tobytes()
        if dumped:
            dumped_at = t
            break
    o.close()
    st.close()
    assert flushed_at is not None and dumped_at == flushed_at
    assert got[3] == 1  # MemTable_count after the flush
    names = sorted(os.listdir("m"))
    assert "6oversize_10_CTB0" in names and len(names) == 1 + 100
    for a, b in (("r0", "q0"), ("r1", "q1"), ("m", "n")):
        assert sorted(os.listdir(a)) == sorted(os.listdir(b))
        for f in os.listdir(a):
            x, y = bytearray(open(os.path.join(a, f), "rb").read()), bytearray(open(os.path.join(b, f), "rb").read())
            assert len(x) == len(y), f
            for lo, hi in _unused_bytes(f):
                x[lo:hi] = y[lo:hi] = bytes(hi - lo)
            assert x == y, f


def _unused_bytes(name):
    """byte ranges of a store file that hold no data: the records' pointer
    fields, which straight_dump fills with its heap addresses (the loaders
    overwrite them), struct padding, and the CTB's own count and time
    fields, which straight_dump never sets (workbench::allocate takes the
    CTB array from malloc, tracing/workbench.cpp:75-82, so they hold
    whatever the heap held)"""
    if "_STcL" in name:   # CTF record: keys, bitmap pointers; tail padding
        return [(16, 32), (76, 80)]
    if "_CTB" in name:    # CTB record: ctfs, count, times, padding, first_widpid .. CTF_capacity,
        return [(0, 32), (32, 72), (76, 104), (120, 128)]  # o_buffer pointers, rtree
    return []
