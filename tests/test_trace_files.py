"""The reference's trace chunk files (tools/datagen.cpp:18-26,
tracing/process.cpp:128-144): glint_trace_write lays steps out as
<prefix><st>_<N>.tr files of 100 steps, and the read-ahead reader
(glint_trace_*) returns every step as written, across chunk boundaries.
Host code only; no device is needed."""
import os

import numpy as np
import pytest

from glint_pipeline_gb300 import GlintError, TraceFiles, write_trace_files
from glint_pipeline_gb300.tracegen import TraceGenerator


def steps(n, count, first=0):
    g = TraceGenerator(0x7777, n, extent_m=3000.0)
    if first:
        g.steps(first)
    return g.steps(count)


def test_chunk_layout_matches_the_reference(tmp_path):
    n = 1000
    pts = steps(n, 230)
    prefix = str(tmp_path / "trace_")
    write_trace_files(prefix, 0, pts)
    for st, count in ((0, 100), (100, 100), (200, 30)):
        path = f"{prefix}{st}_{n}.tr"
        raw = np.fromfile(path, dtype=np.float64)
        assert raw.size == count * n * 2
        np.testing.assert_array_equal(raw.reshape(count, n, 2), pts[st:st + count])


def test_read_ahead_returns_every_step(tmp_path):
    n = 2000
    pts = steps(n, 260)
    prefix = str(tmp_path / "t")
    write_trace_files(prefix, 0, pts)
    tr = TraceFiles(prefix, n, 40, 200, ring=4)
    try:
        prev = None
        for t in range(40, 240):
            cur = tr.step(t)
            np.testing.assert_array_equal(cur, pts[t], err_msg=str(t))
            if prev is not None:   # the step before is still valid
                np.testing.assert_array_equal(prev, pts[t - 1])
            prev = cur
        with pytest.raises(GlintError):
            tr.step(240)           # outside the opened range
    finally:
        tr.close()


def test_write_continues_a_chunk(tmp_path):
    n = 500
    pts = steps(n, 150)
    prefix = str(tmp_path / "c")
    write_trace_files(prefix, 0, pts[:60])
    write_trace_files(prefix, 60, pts[60:])
    raw = np.fromfile(f"{prefix}0_{n}.tr", dtype=np.float64).reshape(100, n, 2)
    np.testing.assert_array_equal(raw, pts[:100])


def test_missing_file_is_reported(tmp_path):
    n = 300
    prefix = str(tmp_path / "m")
    write_trace_files(prefix, 0, steps(n, 100))
    tr = TraceFiles(prefix, n, 90, 20, ring=3)
    try:
        for t in range(90, 100):
            tr.step(t)
        with pytest.raises(GlintError, match="cannot open"):
            tr.step(100)           # the file of steps 100-199 is not there
    finally:
        tr.close()
    assert os.path.exists(f"{prefix}0_{n}.tr")
