"""Contact-trace queries over the flushed store on the GPU against the
oracle's breadth-first restatement over the same meetings."""
import numpy as np
import pytest

from glint_pipeline_gb300 import Configuration, DeviceBench
from oracle.bindings import EDGE_DTYPE, query_bfs
from workloads import case_config, make_points

pytestmark = pytest.mark.gpu


def build_store(name, steps, flush_at, keep=16, host_keep=0):
    box, pts = make_points(name, steps)
    cfgd = case_config(name)
    c = Configuration(num_objects=cfgd["num_objects"], grid_capacity=cfgd["grid_capacity"],
                      grid_amplify=cfgd["grid_amplify"], num_meeting_buckets=cfgd["num_meeting_buckets"],
                      reach_distance=cfgd["reach_distance"], min_meet_time=cfgd["min_meet_time"],
                      schema_update_delay=cfgd["schema_update_delay"], kv_capacity=1 << 22, store_keep=keep,
                      store_host_keep=host_keep)
    g = DeviceBench(c, box, pts[0])
    g.map_box = np.asarray(box, np.float64)
    windows = []   # meetings of each flushed window
    cur = []
    for t in range(steps):
        g.step(pts[t], t)
        cur.append(g.meetings())
        if t in flush_at:
            g.flush()
            windows.append(np.concatenate(cur))
            cur = []
    return g, cfgd["num_objects"], windows


def edges_of(meetings, box=None):
    if box is not None:
        # only meetings whose f32 box lies inside the map become keys
        # (box_contain, cuda/geometry.cu:53-58, 667-670)
        b = meetings["mbr"].astype(np.float64)
        inside = (b[:, 0] >= box[0]) & (b[:, 2] <= box[2]) & (b[:, 1] >= box[1]) & (b[:, 3] <= box[3])
        meetings = meetings[inside]
    e = np.zeros(2 * len(meetings), EDGE_DTYPE)
    e["pid"][0::2], e["target"][0::2] = meetings["pid1"], meetings["pid2"]
    e["pid"][1::2], e["target"][1::2] = meetings["pid2"], meetings["pid1"]
    e["start"][0::2] = e["start"][1::2] = meetings["start"]
    e["end"][0::2] = e["end"][1::2] = meetings["end"]
    return e


def check(g, n, edges, queries):
    got, scanned = g.query(queries)
    assert scanned > 0
    for (seeds, hops, t0, t1), res in zip(queries, got):
        want = query_bfs(edges, n, seeds, hops, t0, t1)
        for h in range(hops):
            np.testing.assert_array_equal(res[h], want[h], err_msg=f"hop {h + 1} of {len(seeds)} seeds, {t0}-{t1}")


def test_query_matches_oracle_bfs():
    g, n, windows = build_store("dense_20k", 50, (20, 35, 49))
    assert g.store_blocks() == 3
    edges = edges_of(np.concatenate(windows), g.map_box)
    rng = np.random.default_rng(3)
    queries = []
    for k, hops, win in [(1, 3, (0, 0)), (10, 2, (0, 0)), (100, 1, (0, 0)), (1000, 3, (0, 0)), (50, 3, (10, 30)),
                         (200, 2, (0, 6)), (30, 3, (40, 50))]:
        seeds = rng.choice(n, k, replace=False).astype(np.uint32)
        queries.append((seeds, hops, win[0], win[1]))
    queries.append((np.array([5, 5, 7, 10 ** 9], np.uint32), 2, 0, 0))  # repeats and an id past N
    check(g, n, edges, queries)
    # a batch larger than one chunk of query slots
    big = [(rng.choice(n, 20, replace=False).astype(np.uint32), 2, 0, 0) for _ in range(70)]
    check(g, n, edges, big)
    g.close()


def test_pull_hops_equal_the_frontier_walk():
    """Once a slot's frontier is at least as large as the set of objects it
    has not reached, the hop runs from the unreached side: each of those
    objects reads its own keys and stops at the first one whose target was
    reached before the hop.  Whole-history and windowed queries whose seeds
    cover most objects (a pull from the first hop), queries that switch at a
    later hop, and every object as a seed all give the oracle's walk."""
    g, n, windows = build_store("dense_20k", 50, (20, 35, 49))
    edges = edges_of(np.concatenate(windows), g.map_box)
    rng = np.random.default_rng(9)
    queries = [(rng.choice(n, k, replace=False).astype(np.uint32), hops, t0, t1) for k, hops, t0, t1 in
               [(15000, 2, 0, 0), (12000, 3, 10, 30), (10000, 2, 40, 49), (3000, 4, 0, 0), (800, 3, 0, 25),
                (n, 1, 0, 0)]]
    check(g, n, edges, queries)
    g.close()


def test_query_over_host_kept_blocks():
    """blocks beyond store_keep move to page-locked host memory (up to
    store_host_keep) and are still queried, read by the GPU over the host
    link; beyond both the oldest block is dropped.  Queries, block reads and
    a compaction over a mix of host- and device-kept blocks agree with the
    oracle and with an all-device context."""
    flush_at = (10, 16, 22, 28, 34, 39)
    g, n, windows = build_store("dense_20k", 40, flush_at, keep=2, host_keep=3)
    assert g.store_blocks() == 5
    edges = edges_of(np.concatenate(windows[1:]), g.map_box)
    rng = np.random.default_rng(6)
    queries = [(rng.choice(n, k, replace=False).astype(np.uint32), hops, 0, 0) for k, hops in
               ((1, 3), (40, 2), (500, 3))] + [(rng.choice(n, 60, replace=False).astype(np.uint32), 2, 12, 30)]
    check(g, n, edges, queries)
    ref, _, _ = build_store("dense_20k", 40, flush_at, keep=5)
    assert ref.store_blocks() == 5
    for i in range(5):
        a, b = g.block(i), ref.block(i)
        for k in ("sids", "keys", "bitmaps", "o_keys"):
            assert np.array_equal(a[k], b[k]), (i, k)
    # serving only: the step state goes, the host-kept blocks move onto the
    # device, queries answer as before and steps are refused
    got_before, _ = g.query(queries)
    assert g.serve_only(reserve=1 << 30) == 5
    got_after, _ = g.query(queries)
    for a, b in zip(got_before, got_after):
        for h in range(len(a)):
            np.testing.assert_array_equal(a[h], b[h])
    box, pts = make_points("dense_20k", 41)
    with pytest.raises(Exception):
        g.step(pts[40], 40)
    info_g = g.compact(0, 5, 4)
    info_r = ref.compact(0, 5, 4)
    assert info_g["kv_count"] == info_r["kv_count"]
    for k in ("sids", "keys", "bitmaps", "o_keys"):
        assert np.array_equal(g.block(0)[k], ref.block(0)[k]), k
    g.close()
    ref.close()


def test_query_kept_blocks_only():
    g, n, windows = build_store("dense_20k", 40, (12, 25, 39), keep=2)
    assert g.store_blocks() == 2
    edges = edges_of(np.concatenate(windows[1:]), g.map_box)
    rng = np.random.default_rng(4)
    check(g, n, edges, [(rng.choice(n, 300, replace=False).astype(np.uint32), 3, 0, 0)])
    g.close()


def test_serving_mix_equals_alone():
    """Continuous batching: queries admitted while others are in flight, with
    fewer slots than queries, give exactly their results alone (and the
    oracle's)."""
    from glint_pipeline_gb300 import Server
    g, n, windows = build_store("dense_20k", 50, (20, 35, 49))
    edges = edges_of(np.concatenate(windows), g.map_box)
    rng = np.random.default_rng(9)
    queries = []
    for i in range(30):
        k = int(np.exp(rng.uniform(0, np.log(1000))))
        hops = int(rng.integers(1, 4))
        if i % 3 == 0:
            win = (0, 0)
        else:
            t0 = int(rng.integers(0, 45))
            win = (t0, t0 + int(rng.integers(2, 30)))
        queries.append((rng.choice(n, k, replace=False).astype(np.uint32), hops, win[0], win[1]))
    alone = [g.query([q])[0][0] for q in queries]
    srv = Server(g, max_slots=7)
    assert srv.slots == 7
    tickets = {}
    pending = list(range(len(queries)))
    results = {}
    step = 0
    while pending or len(results) < len(queries):
        for _ in range(int(rng.integers(0, 5))):   # arrivals between steps
            if pending:
                i = pending.pop(0)
                tickets[srv.submit(*queries[i])] = i
        active, queued = srv.step()
        for t, i in list(tickets.items()):
            r = srv.poll(t)
            if r is not None:
                results[i] = r[0]
                del tickets[t]
        step += 1
        assert step < 10_000
    for i, (seeds, hops, t0, t1) in enumerate(queries):
        want = query_bfs(edges, n, seeds, hops, t0, t1)
        for h in range(hops):
            np.testing.assert_array_equal(results[i][h], alone[i][h], err_msg=f"query {i} hop {h + 1} (mix vs alone)")
            np.testing.assert_array_equal(results[i][h], want[h], err_msg=f"query {i} hop {h + 1} (vs oracle)")
    srv.close()
    g.close()


def test_store_files_round_trip(tmp_path, monkeypatch):
    """glint_store_dump writes the last flushed block in the reference's file
    layout, byte for byte what glint_store_write makes of the same block read
    to the host; glint_store_load of those files into a fresh context answers
    queries as the oracle does over that window's meetings."""
    import os
    from glint_pipeline_gb300 import write_store_files
    monkeypatch.chdir(tmp_path)
    for d in ("r0", "r1", "m", "h0", "h1", "hm"):
        os.makedirs(d)
    g, n, windows = build_store("dense_20k", 40, (20, 39), keep=1)
    g.dump_store("r", "m", "6oversize_3600", 1)
    store = g.store()
    write_store_files(store, store["info"], n, "h", "hm", "6oversize_3600", 1)
    names = sorted(os.listdir("m"))
    assert len(names) == 1 + store["ctfs"].shape[0]
    for name in names:
        assert open(f"m/{name}", "rb").read() == open(f"hm/{name}", "rb").read(), name
    for i in range(store["ctfs"].shape[0]):
        a = open(f"r{i % 2}/6oversize_3600_SSTable_1-{i}", "rb").read()
        assert a == open(f"h{i % 2}/6oversize_3600_SSTable_1-{i}", "rb").read()
    box = g.map_box
    cfg = g.config
    g.close()
    f = DeviceBench(cfg, box, make_points("dense_20k", 1)[1][0])
    try:
        f.load_store("r", "m", "6oversize_3600", 1)
        assert f.store_blocks() == 1
        edges = edges_of(windows[-1], box)
        rng = np.random.default_rng(9)
        queries = [(rng.choice(n, k, replace=False).astype(np.uint32), hops, t0, t1)
                   for k, hops, t0, t1 in [(1, 3, 0, 0), (100, 2, 0, 0), (1000, 3, 0, 0), (50, 2, 24, 34)]]
        check(f, n, edges, queries)
        with pytest.raises(Exception):
            f.load_store("r", "m", "6oversize_3600", 7)   # no such block
    finally:
        f.close()
