"""Host logic of bench.py (no GPU): the byte model and roofline fields of the
JSON line, the latency summary of the serving leg, and the L2 note."""
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)


@pytest.fixture(scope="module")
def bench():
    argv = sys.argv
    sys.argv = ["bench.py"]
    try:
        import bench as b
        yield b
    finally:
        sys.argv = argv


def _form(N, contacts, meetings, ms):
    stage = {k: 0.0 for k in ("copy", "partition", "filter", "refine", "insert", "identify", "schema", "total")}
    stage.update(refine=ms["refine"], identify=ms["identify"], insert=ms["insert"], total=ms["total"])
    per = {"contacts": contacts, "meetings": meetings, "new_keys": 0, "checks": 0, "cross_checks": 0,
           "border_objects": 0, "buckets": 1 << 30, "expired": 0}
    return {"stage_ms": stage, "per_step": per, "ms_per_step": ms["total"]}


def test_byte_model(bench):
    N, P, M = 10_000_000, 200_000_000, 6_000_000
    total, by = bench.step_bytes_8d(N, {"contacts": P, "meetings": M})
    assert total == 40 * N + 32 * P + 48 * M
    assert by["refine"] == 16 * N + 32 * P
    assert by["partition"] + by["refine"] + by["identify"] == total


def test_roofline_is_on_refine_and_follows_the_model(bench):
    N, P, M = 10_000_000, 200_000_000, 6_000_000
    # identify slower than refine: the roofline still reports refine's kernel
    f = _form(N, P, M, {"refine": 11.0, "identify": 12.0, "insert": 5.0, "total": 36.0})
    r = bench.roofline(f, N, 1 << 30, "tuned")
    assert r["kernel"] == "k_refine_fp32" and r["kernel_stage"] == "refine"
    assert r["slowest_stage"] == "identify"
    by = 16 * N + 32 * P
    assert r["algorithmic_bytes"] == by
    assert r["achieved"] == pytest.approx(by / 0.011 / 1e9)
    assert r["frac"] == pytest.approx(r["achieved"] / r["peak"])
    assert r["frac_step"] == pytest.approx((40 * N + 32 * P + 48 * M) / 0.036 / 1e9 / r["peak"])
    assert r["frac_step_with_flush"] > r["frac_step"]
    assert r["traffic"] == bench.TRAFFIC_10M_2P30["refine"]
    assert bench.roofline(f, N, 1 << 30, "plain")["kernel"] == "k_refine_fp64"
    # the ncu traffic figure belongs to the 10M, 2^30-bucket tuned workload only
    assert bench.roofline(f, 2_000_000, 1 << 26, "tuned")["traffic"] is None


def test_latency_summary(bench):
    lat = np.arange(1, 101, dtype=np.float64)
    out = bench.latency_summary(lat, 100, 0, 20.0)
    assert out["finished"] == 100 and out["p50_ms"] == pytest.approx(np.percentile(lat, 50))
    # unfinished queries rank after every finished one: p99 is null past them
    out = bench.latency_summary(lat[:97], 100, 3, 20.0)
    assert out["finished"] == 97 and out["p50_ms"] == 50.0 and out["p99_ms"] is None


def test_l2_note(bench):
    args = bench.parse()
    assert bench.workload_config(args, 10_000_000, "tuned")["l2"].startswith("inputs larger than L2")
    args.buckets = 1 << 20
    assert "fits in L2" in bench.workload_config(args, 100_000, "tuned")["l2"]
