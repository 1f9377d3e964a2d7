"""Golden digests of the reference's OWN GPU key generation, active
multi-search and flush (cuda/geometry.cu: cuda_identify_meetings and the
"4.5 cuda sort" block of process_with_gpu, run from the reference's
unmodified sources compiled into oracle/_ref/geometry.cubin by
oracle/build_ref.sh, through oracle/ref_gpu_driver.cpp).

Needs a GPU and the cubin; writes ref_gpu_flush.npz (default: next to this
script).  The inputs are the oracle's meetings on seeded workloads, so the
digests pin the oracle's flush restatement and the device flush to the
reference's own kernels:

    python tests/golden/make_ref_gpu_golden.py [out.npz]
"""
from __future__ import annotations

import hashlib
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from workloads import case_config, make_points  # noqa: E402

# name -> (steps, flush steps, dProbFalse, max_meet_time, split_num)
FLUSH_CASES = {
    "dense_20k": (50, (20, 35, 49), 100.0, 4096, 10),
    "dense_20k_oversize": (40, (25, 39), 2e-9, 4096, 10),
    "small_100k": (60, (30, 59), 100.0, 4096, 10),
    "collide_20k": (45, (44,), 100.0, 4096, 4),
}
SEARCH_CASES = {"dense_20k": (24, 400), "reach_8k": (20, 300)}
FIELDS = ("keys", "sids", "ctf_capacity", "ctfs", "bitmaps", "o_keys", "o_boxes", "o_bitmap")
INFO = ("kv_count", "key_bytes", "oversize_kv_count", "oversize_start_time_min", "oversize_start_time_max",
        "oversize_end_time_min", "oversize_end_time_max", "sid_count", "oversize_oid_count")


def workload(case):
    return case.replace("_oversize", "")


def digest(a) -> str:
    return hashlib.sha256(np.ascontiguousarray(a).view(np.uint8).tobytes()).hexdigest()


def flush_digests(r) -> list[str]:
    return [digest(r[f]) for f in FIELDS]


def info_tuple(info) -> list[int]:
    return [int(getattr(info, f)) for f in INFO]


def search_pids(case, t):
    n = case_config(case)["num_objects"]
    rng = np.random.default_rng(1000 + t)
    return np.sort(rng.choice(n, SEARCH_CASES[case][1], replace=False)).astype(np.uint32)


def canonical_search(rec):
    """records as a multiset: sorted by (pid, target, start, end)"""
    r = np.ascontiguousarray(rec)
    order = np.lexsort((r["end"], r["start"], r["target"], r["pid"]))
    return r[order]


def run_flush_case(case, store_cls, run_ref=True):
    """the oracle's meetings of every step through the reference's kernels
    (run_ref) and the oracle's restatement; per flush: digests and info"""
    from oracle.bindings import Oracle, RefGpu, cantor_inverse, make_config
    steps, flush_at, dprob, max_meet, split = FLUSH_CASES[case]
    name = workload(case)
    box, pts = make_points(name, steps)
    cfgd = case_config(name)
    o = Oracle(make_config(**cfgd), box, pts[0])
    kw = dict(max_meet_time=max_meet, dProbFalse=dprob, kv_capacity=1 << 22, CTF_count=split * split,
              split_num=split)
    st = store_cls(cfgd["num_objects"], box, first_end_time_min=cfgd["min_meet_time"], **kw)
    rg = RefGpu(cfgd["num_objects"], box, min_meet_time=cfgd["min_meet_time"], **kw) if run_ref else None
    etm = cfgd["min_meet_time"]
    out = []
    for t in range(steps):
        o.step(pts[t], t)
        mo = o.meetings()
        rec = np.zeros(mo.shape[0], np.dtype([("pid1", "<u4"), ("pid2", "<u4"), ("start", "<u4"), ("end", "<u4"),
                                              ("mbr", "<f4", (4,))]))
        rec["pid1"], rec["pid2"] = cantor_inverse(mo["key"])
        rec["start"], rec["end"], rec["mbr"] = mo["start"], mo["end"], mo["mbr"]
        st.add_meetings(rec)
        if rg is not None:
            rg.identify(mo, t, etm)
        if t in flush_at:
            rc, oi = st.flush(t)
            assert rc == 0, f"{case}: oracle flush at {t} outside the reference's domain"
            assert oi.bits_outside == 0
            ora = st.result(oi)
            ref = rg.flush(t) if rg is not None else None
            out.append({"t": t, "oracle": ora, "oracle_info": oi, "ref": ref})
            etm = t
    o.close()
    st.close()
    if rg is not None:
        rg.close()
    return out


def main():
    from oracle.bindings import Oracle, RefGpu, Store, make_config
    path = sys.argv[1] if len(sys.argv) > 1 else os.path.join(HERE, "ref_gpu_flush.npz")
    data = {}
    for case in FLUSH_CASES:
        res = run_flush_case(case, Store)
        data[f"{case}/flush_steps"] = np.array([r["t"] for r in res], np.uint32)
        data[f"{case}/digests"] = np.array([flush_digests(r["ref"]) for r in res])
        data[f"{case}/info"] = np.array([info_tuple(r["ref"]["info"]) for r in res], np.uint64)
        data[f"{case}/bits_in_slack"] = np.array([int(r["ref"]["info"].bits_in_slack) for r in res], np.uint64)
        same = [flush_digests(r["ref"]) == flush_digests(r["oracle"]) for r in res]
        print(case, "flushes", len(res), "oracle equal", same, flush=True)
    for case, (steps, _) in SEARCH_CASES.items():
        box, pts = make_points(case, steps)
        cfgd = case_config(case)
        o = Oracle(make_config(**cfgd), box, pts[0])
        digs, counts = [], []
        for t in range(steps):
            o.step(pts[t], t)
            if t < 8:
                continue
            k, s, e, m = o.buckets()
            occ = k != (1 << 62)
            table = np.zeros(int(occ.sum()), np.dtype([("key", "<u8"), ("start", "<u4"), ("end", "<u4"),
                                                       ("mbr", "<f4", (4,))]))
            table["key"], table["start"], table["end"], table["mbr"] = k[occ], s[occ], e[occ], m[occ]
            rg = RefGpu(cfgd["num_objects"], box, min_meet_time=cfgd["min_meet_time"])
            got = canonical_search(rg.identify(table, t, cfgd["min_meet_time"], search_pids(case, t)))
            rg.close()
            want = canonical_search(o.active_search(search_pids(case, t)))
            print(case, t, len(got), "oracle equal", got.tobytes() == want.tobytes(), flush=True)
            digs.append(digest(got))
            counts.append(len(got))
        data[f"search/{case}/digests"] = np.array(digs)
        data[f"search/{case}/counts"] = np.array(counts, np.uint64)
        o.close()
    np.savez(path, **data)
    print("wrote", path)


if __name__ == "__main__":
    main()
