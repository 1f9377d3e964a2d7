"""The CPU oracle (oracle/glint_oracle.c) against the reference's own output.

Pinned two ways: against fixtures in tests/golden generated by running the
reference's sources (tests/golden/make_golden.py), and - on machines that
hold the reference sources - step by step against a fresh build of them,
including the schema, both free stacks and the whole bucket table.
"""
import os

import numpy as np
import pytest

from oracle.bindings import Oracle, Reference, make_config, ref_available
from workloads import CASES, case_config, digest, make_points

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def golden(name):
    return np.load(os.path.join(GOLDEN, f"{name}.npz"))


@pytest.mark.parametrize("name", sorted(CASES))
def test_generator_inputs_pinned(name):
    box, pts = make_points(name)
    assert digest(pts[0], pts[-1]) == str(golden(name)["points_digest"])


@pytest.mark.parametrize("name", [n for n in sorted(CASES) if n != "small_100k"])
def test_oracle_matches_golden(name):
    g = golden(name)
    box, pts = make_points(name)
    o = Oracle(make_config(**case_config(name)), box, pts[0])
    bounds = g["bounds"]
    for t in range(pts.shape[0]):
        o.step(pts[t], t)
        m = o.meetings()
        c = o.counts()
        a, b = bounds[t], bounds[t + 1]
        np.testing.assert_array_equal(m["key"], g["keys"][a:b], err_msg=f"step {t}")
        np.testing.assert_array_equal(m["start"], g["starts"][a:b])
        np.testing.assert_array_equal(m["end"], g["ends"][a:b])
        assert (c.grid_check_counter, c.kv_count, c.num_taken_buckets, c.num_active_meetings, c.grids_stack_index,
                c.schema_stack_index) == tuple(int(v) for v in g["counts"][t]), f"step {t}"
        assert digest(m["key"], m["start"], m["end"]) == str(g["step_digests"][t])
    sch, ss, gs, gc = o.schema()
    valid = sch["type"] != 0
    assert digest(sch["type"], sch["grid_id"][valid], sch["level"][valid], sch["mid_x"][valid], sch["mid_y"][valid],
                  sch["low"][valid], sch["high"][valid]) == str(g["schema_digest"])
    c = o.counts()
    assert digest(ss[c.schema_stack_index:], gs[c.grids_stack_index:]) == str(g["stacks_digest"])
    bk, bs, be, bm = o.buckets()
    occ = bk != (1 << 62)
    assert digest(bk, bs[occ]) == str(g["buckets_digest"])
    o.close()


def test_oracle_matches_golden_small_100k():
    """The small plain case: 100k objects x 100 steps, per-step digests."""
    g = golden("small_100k")
    box, pts = make_points("small_100k")
    o = Oracle(make_config(**case_config("small_100k")), box, pts[0])
    for t in range(pts.shape[0]):
        o.step(pts[t], t)
        m = o.meetings()
        assert digest(m["key"], m["start"], m["end"]) == str(g["step_digests"][t]), f"step {t}"
    o.close()


@pytest.mark.skipif(not ref_available(), reason="reference sources not on this machine")
@pytest.mark.parametrize("seed,n,steps,ext,B,extra", [
    (0xABC1, 12_000, 30, 3000.0, 17011, {}),
    (0xABC2, 6_000, 30, 1500.0, 0, {"grid_capacity": 10}),
    (0xABC3, 9_000, 25, 2500.0, 0, {"schema_update_delay": 3, "grid_capacity": 30}),
])
def test_oracle_matches_reference_build(seed, n, steps, ext, B, extra):
    from glint_pipeline_gb300.tracegen import TraceGenerator
    g = TraceGenerator(seed, n, 0, extent_m=ext)
    box, pts = g.box(), g.steps(steps)
    cfg = make_config(n, num_meeting_buckets=B or 2 * n, **extra)
    o, r = Oracle(cfg, box, pts[0]), Reference(cfg, box, pts[0])
    for t in range(steps):
        o.step(pts[t], t)
        r.step(pts[t], t)
        mo, mr = o.meetings(), r.meetings()
        np.testing.assert_array_equal(mo["key"], mr["key"])
        np.testing.assert_array_equal(mo["start"], mr["start"])
        np.testing.assert_array_equal(mo["end"], mr["end"])
        ko, so, eo, _ = o.buckets()
        kr, sr, er = r.buckets()
        np.testing.assert_array_equal(ko, kr)
        occ = kr != (1 << 62)
        np.testing.assert_array_equal(so[occ], sr[occ])
        np.testing.assert_array_equal(eo[occ], er[occ])
    so_, sso, gso, gco = o.schema()
    sr_, ssr, gsr, gcr = r.schema()
    np.testing.assert_array_equal(so_["type"], sr_["type"])
    v = so_["type"] != 0
    for f in ("grid_id", "level", "mid_x", "mid_y", "low", "high"):
        np.testing.assert_array_equal(so_[f][v], sr_[f][v])
    np.testing.assert_array_equal(sso, ssr)
    np.testing.assert_array_equal(gso, gsr)


def test_sin_cr_is_correctly_rounded():
    mpmath = pytest.importorskip("mpmath")
    from oracle.bindings import oracle_lib
    lib = oracle_lib()
    mpmath.mp.prec = 160
    rng = np.random.default_rng(7)
    xs = np.concatenate([rng.random(3000) * 1.5707963, 0.838 + rng.random(3000) * 0.008])
    for x in xs:
        assert lib.go_sin_cr(float(x)) == float(mpmath.sin(mpmath.mpf(float(x))))


def _search_restated(keys, starts, ends, mbrs, cur, min_meet, pids, n_objects):
    """numpy restatement of the active multi-search (cuda/geometry.cu:605-663)."""
    from oracle.bindings import SEARCH_DTYPE, cantor_inverse
    listed = np.zeros(n_objects, bool)
    listed[np.asarray(pids)[np.asarray(pids) < n_objects]] = True
    occ = (keys != (1 << 62)) & (ends == cur) & ((cur - starts.astype(np.int64)) >= min_meet + 1)
    idx = np.nonzero(occ)[0]
    a, b = cantor_inverse(keys[idx])
    rows = []
    for j, s in enumerate(idx):
        for p, q in ((a[j], b[j]), (b[j], a[j])):
            if listed[p]:
                rows.append((p, q, starts[s], ends[s], mbrs[s]))
    out = np.zeros(len(rows), SEARCH_DTYPE)
    for i, r in enumerate(rows):
        out[i] = r
    return out


def test_oracle_active_search_restated():
    """The oracle's active search equals a direct restatement over its buckets."""
    box, pts = make_points("dense_20k", 20)
    cfgd = case_config("dense_20k")
    o = Oracle(make_config(**cfgd), box, pts[0])
    rng = np.random.default_rng(7)
    for t in range(pts.shape[0]):
        o.step(pts[t], t)
        if t < 8:
            continue
        pids = np.concatenate([rng.choice(cfgd["num_objects"], 400, replace=False), [0, 0, 10**9]]).astype(np.uint32)
        got = o.active_search(pids)
        k, s, e, m = o.buckets()
        want = _search_restated(k, s, e, m, t, cfgd["min_meet_time"], pids, cfgd["num_objects"])
        assert len(want) > 0
        np.testing.assert_array_equal(got.view(np.uint8), want.view(np.uint8))
    o.close()


@pytest.mark.parametrize("name,threads", [("collide_20k", 7), ("skew_5k", 3), ("delay_10k", 16), ("dense_20k", 5)])
def test_threaded_oracle_equals_single_thread(name, threads):
    """Host threads change no result: meetings, counts, schema, stacks and the
    whole bucket table equal the single-threaded run step by step (prime
    buckets at high load, leaf overflow drops, delayed schema updates)."""
    box, pts = make_points(name, 30)
    cfg = make_config(**case_config(name))
    one, many = Oracle(cfg, box, pts[0]), Oracle(cfg, box, pts[0], threads=threads)
    reruns = 0
    for t in range(pts.shape[0]):
        one.step(pts[t], t)
        many.step(pts[t], t)
        np.testing.assert_array_equal(one.meetings().view(np.uint8), many.meetings().view(np.uint8),
                                      err_msg=f"step {t}")
        c1, c2 = one.counts(), many.counts()
        fields = [f for f, _ in c1._fields_ if f != "range_reruns"]
        assert [getattr(c1, f) for f in fields] == [getattr(c2, f) for f in fields]
        reruns += c2.range_reruns
        if t % 6 == 5:
            for a, b in zip(one.buckets(), many.buckets()):
                np.testing.assert_array_equal(a, b)
    for a, b in zip(one.schema(), many.schema()):
        np.testing.assert_array_equal(a.view(np.uint8), b.view(np.uint8))
    if name in ("collide_20k", "skew_5k"):
        # high load: probes do run off the end of a slot range and are handed on
        assert reruns > 0
    one.close()
    many.close()


@pytest.mark.skipif(not ref_available(), reason="the reference's sources are not on this machine")
def test_calibration_script(tmp_path):
    """oracle/calibrate_cpu.py times the reference's own CPU stages (-O2 and
    as shipped) and the oracle on one host; on one thread all three report
    the same meetings."""
    import json
    import subprocess
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    out = tmp_path / "calibration.md"
    r = subprocess.run([sys.executable, os.path.join(root, "oracle", "calibrate_cpu.py"), "--objects", "20000",
                        "--buckets", "65536", "--steps", "2", "--warmup", "6", "--out", str(out)],
                       capture_output=True, text=True, timeout=900)
    assert r.returncode == 0, r.stderr[-2000:]
    rows = [json.loads(line) for line in r.stdout.splitlines() if line.startswith("{")]
    one = {row["label"]: row["meetings"] for row in rows if row["threads"] == 1}
    assert set(one) == {"reference -O2", "reference as shipped (-g)", "port (oracle, -O2)"}
    assert len(set(one.values())) == 1 and next(iter(one.values())) > 0
    text = out.read_text()
    assert "| reference -O2 | 1 |" in text and "| port (oracle, -O2) | 1 |" in text
