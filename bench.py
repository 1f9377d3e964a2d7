"""Benchmark: object-timesteps/s of the contact-tracing step at 10M objects.

Workload (BASELINE configs[1]): the seeded Manhattan-grid generator, 10M
objects, FP64 lon/lat, reach 2 m, minimum meeting 5 steps, QuadTree leaf
capacity 50 (the reference default), a meeting table of 2^30 buckets.  One
step = partition -> filter -> refine -> table insert -> identify -> schema
update for one 1-second timestep of all objects.  Both forms produce
bit-identical meetings; "plain" runs the reference's FP64 test on every
candidate pair, "tuned" screens pairs in FP32 with a guard band first.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]
                    [--objects N] [--mode both|plain|tuned]

value: device-resident inputs (every step's points generated on the device
beforehand), the K timed steps measured with CUDA events on the step's
stream.  e2e: further steps through glint_step() with points in pinned host
memory (host->device copy inside the timed region) and each step's meetings
copied back.  Under torchrun (N>1) every rank runs an independent replica on
its own GPU (the path has no data exchange): the slowest rank's time counts
and value sums all ranks' object-timesteps.
"""
from __future__ import annotations

import argparse
import ctypes
import glob
import json
import os
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "object-timesteps/s at 10M objs, bit-exact meetings, plain vs tuned; query p50/p99"
UNIT = "object-timesteps/s"
STAGES = ["copy", "partition", "filter", "refine", "insert", "identify", "schema", "total"]


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=20)
    p.add_argument("--warmup", type=int, default=8)
    p.add_argument("--impl", default="glint", choices=["glint", "reference"])
    p.add_argument("--objects", type=int, default=10_000_000)
    p.add_argument("--buckets", type=int, default=1 << 30)
    p.add_argument("--mode", default="both", choices=["both", "plain", "tuned"])
    p.add_argument("--e2e-steps", type=int, default=8)
    p.add_argument("--no-e2e", action="store_true", help="skip the host-buffer pass (profiling runs)")
    p.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline (profiling runs)")
    p.add_argument("--cpu-sample-objects", type=int, default=1_000_000)
    p.add_argument("--cpu-sample-steps", type=int, default=3)
    return p.parse_args()


def dist_init():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    pg = None
    if world > 1:
        import torch.distributed as dist
        os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
        dist.init_process_group("gloo", rank=rank, world_size=world)
        pg = dist
    return rank, world, local, pg


def barrier(pg):
    if pg is not None:
        pg.barrier()


def allreduce_max(pg, v):
    if pg is None:
        return v
    import torch
    t = torch.tensor([float(v)], dtype=torch.float64)
    pg.all_reduce(t, op=pg.ReduceOp.MAX)
    return float(t.item())


class Clocks:
    """nvidia-smi samples of SM clock and throttle reasons during a timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device, tag):
        self.device = device
        self.proc = None
        self.path = os.path.join(ROOT, "gpurun_out", f"clocks_{tag}_{os.getpid()}.csv")

    def __enter__(self):
        try:
            os.makedirs(os.path.dirname(self.path), exist_ok=True)
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "100"], stdout=self.f,
                                         stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()
            self.f.close()

    def summary(self):
        out = {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        try:
            rows = [[c.strip() for c in r.split(",")] for r in open(self.path).read().strip().splitlines() if r.strip()]
        except Exception:
            return out
        rows = [r for r in rows if len(r) >= 9]
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        if sm:
            out["sm_mhz"] = float(np.median(sm))
            out["sm_max_mhz"] = float(rows[0][2]) if rows[0][2].replace(".", "").isdigit() else None
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = set()
        for r in rows:
            for k, name in enumerate(names):
                if r[5 + k] == "Active":
                    reasons.add(name)
        out["reasons"] = sorted(reasons)
        out["samples"] = len(rows)
        return out


def peaks():
    try:
        return json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except Exception:
        return {}


def cudart():
    for cand in ["libcudart.so", "libcudart.so.13"] + glob.glob("/usr/local/cuda/lib64/libcudart.so*"):
        try:
            lib = ctypes.CDLL(cand)
            lib.cudaMemcpy.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t, ctypes.c_int]
            lib.cudaFree.argtypes = [ctypes.c_void_p]
            lib.cudaFreeHost.argtypes = [ctypes.c_void_p]
            return lib
        except OSError:
            continue
    raise OSError("libcudart not found")


def stage_bytes(stage, N, st, K):
    """Algorithmic bytes of one launch of a stage's main kernel."""
    if stage == "refine":
        # member tiles x, y, L, id (28 B/object); per cross check the querier's
        # x, y, L and the check (32 B); per contact one table record read
        # (32 B), its box written back (16 B) and its stamp (1 B); per new pair
        # a 16 B new-list entry
        return 28 * N + 32 * st["cross_checks"] + 49 * st["contacts"] + 16 * st["new_keys"]
    if stage == "identify":
        # two stamp passes (2 B/bucket), per expiring entry its 16 B head read
        # and 8 B write, per reported meeting the record (32 B) and log entry (32 B)
        return 2 * st["buckets"] + 24 * st["expired"] + 64 * st["meetings"]
    if stage == "filter":
        # per object its leaf/last_valid/count (12 B); per border object its
        # point and L (24 B); per check 8 B by querier + 8 B by target
        return 12 * N + 24 * st["border_objects"] + 16 * st["cross_checks"]
    if stage == "insert":
        # per new pair: list entry (16 B), record head CAS (32 B), stamp, then
        # the finalize pass (16 B list + 32 B record + 32 B of points)
        return 129 * st["new_keys"]
    if stage == "partition":
        # points (16 B) + leaf/last_valid/leaf node/L writes (20 B) + scatter (8 B)
        # + gather (16+8+4 B in, 28 B out)
        return 100 * N
    return 0


def run_form(args, mode, N, local, pg, world, box, first, pb, ob, dbuf, step_bytes, rt):
    import glint_pipeline_gb300 as gp
    from glint_pipeline_gb300 import _abi
    from glint_pipeline_gb300.tracegen import SEED_SCALE, TraceGenerator
    lib = _abi.lib()
    K, W = args.steps, max(args.warmup, 3)
    cfg = gp.Configuration(num_objects=N, num_meeting_buckets=args.buckets, device=local, timing=True,
                           precision_mode=1 if mode == "tuned" else 0)
    bench = gp.DeviceBench(cfg, box, first)
    for t in range(W):
        bench.step_device(dbuf.value + t * step_bytes, t)
        bench.sync()
    barrier(pg)
    stage_ms = np.zeros(8)
    acc = {"candidates": 0, "contacts": 0, "new_keys": 0, "meetings": 0, "cross_checks": 0, "border_objects": 0,
           "taken": 0, "active": 0, "band_pairs": 0, "rechecks": 0, "ambiguous": 0}
    launches = 0
    dev_ms = 0.0
    last = None
    with Clocks(local, mode) as clk:
        for t in range(W, W + K):
            bench.step_device(dbuf.value + t * step_bytes, t)
            st = bench.sync()
            stage_ms += np.array(st.ms)
            dev_ms += st.ms[7]
            launches += st.launches
            acc["candidates"] += st.candidates
            acc["contacts"] += st.contacts
            acc["new_keys"] += st.new_keys
            acc["meetings"] += st.meetings
            acc["cross_checks"] += st.cross_checks
            acc["border_objects"] += st.border_objects
            acc["taken"] += st.num_taken_buckets
            acc["active"] += st.num_active_meetings
            acc["band_pairs"] += st.band_pairs
            acc["rechecks"] += st.rechecks
            acc["ambiguous"] += st.ambiguous
            last = st
    dev_s = allreduce_max(pg, dev_ms / 1000.0)
    per = {k: v / K for k, v in acc.items()}
    per["buckets"] = args.buckets
    per["expired"] = per["taken"] - per["active"]
    per["checks"] = last.checks
    per["leaves"] = last.leaves
    per["error_flags"] = last.error_flags
    out = {"value": N * K * world / dev_s, "ms_per_step": 1000.0 * dev_s / K,
           "stage_ms": {k: v / K for k, v in zip(STAGES, stage_ms)}, "per_step": per,
           "clocks": clk.summary(), "gpu_launches": launches}

    if args.no_e2e:
        out["e2e"] = None
        bench.close()
        return out
    # e2e: continue the trajectory with host-resident points
    ke = max(1, min(args.e2e_steps, K))
    base = W + K
    hbuf = ctypes.c_void_p()
    assert rt.cudaMallocHost(ctypes.byref(hbuf), ctypes.c_size_t(step_bytes * ke)) == 0
    gh = ctypes.c_void_p()
    g3 = TraceGenerator(SEED_SCALE, N)
    assert lib.glint_gen_create(g3.params_bytes(), len(pb), g3.objects_bytes(), N, len(ob) // N, 0,
                                ctypes.byref(gh)) == 0
    tmp = ctypes.c_void_p()
    assert rt.cudaMalloc(ctypes.byref(tmp), ctypes.c_size_t(step_bytes)) == 0
    for t in range(base + ke):
        lib.glint_gen_step(gh, tmp, ctypes.c_void_p(bench.stream))
        if t >= base:
            rt.cudaDeviceSynchronize()
            rt.cudaMemcpy(ctypes.c_void_p(hbuf.value + (t - base) * step_bytes), tmp, ctypes.c_size_t(step_bytes), 2)
    rt.cudaDeviceSynchronize()
    lib.glint_gen_destroy(gh)
    rt.cudaFree(tmp)
    arr = (ctypes.c_double * (2 * N * ke)).from_address(hbuf.value)
    host = np.frombuffer(arr, dtype=np.float64).reshape(ke, N, 2)
    barrier(pg)
    d2h = 0
    t0 = time.perf_counter()
    for k in range(ke):
        bench.step(host[k], base + k)
        m = bench.meetings()
        d2h += m.nbytes + ctypes.sizeof(_abi.GlintStepStats)
    dt = allreduce_max(pg, time.perf_counter() - t0)
    out["e2e"] = {"value": N * ke * world / dt, "unit": UNIT, "h2d_bytes_per_step": step_bytes,
                  "d2h_bytes_per_step": int(d2h / ke), "steps": ke}
    del host, arr
    rt.cudaFreeHost(hbuf)
    bench.close()
    return out


def roofline(form, N):
    pk = peaks()
    hbm = pk.get("hbm_gbs")
    stages = {k: v for k, v in form["stage_ms"].items() if k in ("partition", "filter", "refine", "insert", "identify")}
    top = max(stages, key=stages.get)
    ms = stages[top]
    by = stage_bytes(top, N, form["per_step"], 1)
    achieved = by / (ms / 1000.0) / 1e9 if ms > 0 else None
    peak = hbm if hbm else 6800.0
    return {"kernel_stage": top, "bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
            "frac": achieved / peak if achieved else None, "traffic": None, "algorithmic_bytes": by,
            "peak_source": "of measured (MEASURED_PEAKS.json hbm_gbs)" if hbm else "of fallback"}


def cpu_baseline(args):
    """The CPU oracle (C restatement of the reference's stages) on a bounded sample."""
    from glint_pipeline_gb300.tracegen import SEED_SCALE, TraceGenerator
    from oracle.bindings import Oracle, make_config
    n, k = args.cpu_sample_objects, args.cpu_sample_steps
    g = TraceGenerator(SEED_SCALE, n)
    box, pts = g.box(), g.steps(k + 1)
    o = Oracle(make_config(n, num_meeting_buckets=1 << 24), box, pts[0])
    o.step(pts[0], 0)
    t0 = time.perf_counter()
    for t in range(1, k + 1):
        o.step(pts[t], t)
    dt = time.perf_counter() - t0
    o.close()
    return {"value": n * k / dt, "unit": UNIT, "cores": 1, "kind": "port",
            "sample": f"{n} objects of the same generator (seed, box, hotspots), {k} timed steps after one; "
                      f"single-threaded C restatement of the reference's CPU stages (-O2)"}


def run_reference_arm(args, rank, world, pg):
    if rank != 0:
        return
    from glint_pipeline_gb300.tracegen import SEED_SCALE, TraceGenerator
    from oracle.bindings import Oracle, make_config
    n = args.cpu_sample_objects
    g = TraceGenerator(SEED_SCALE, n)
    steps = max(1, min(args.steps, 5))
    warm = max(1, min(args.warmup, 3))
    box, pts = g.box(), g.steps(warm + steps)
    o = Oracle(make_config(n, num_meeting_buckets=1 << 24), box, pts[0])
    for t in range(warm):
        o.step(pts[t], t)
    t0 = time.perf_counter()
    for t in range(warm, warm + steps):
        o.step(pts[t], t)
    dt = time.perf_counter() - t0
    value = n * steps / dt
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
            "steps": steps, "warmup": warm, "ms_per_step": 1000 * dt / steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": f"Manhattan-grid generator (configs[1] generator), {n}-object sample, reach 2 m, "
                                   f"min meeting 5, leaf capacity 50", "objects": n},
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": 1, "kind": "port",
                             "sample": f"{n} objects x {steps} steps; the reference's sources are not on this "
                                       f"machine, so its CPU stages run as the single-threaded C restatement"},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def main():
    args = parse()
    rank, world, local, pg = dist_init()
    if args.impl == "reference":
        run_reference_arm(args, rank, world, pg)
        return
    from glint_pipeline_gb300 import _abi
    from glint_pipeline_gb300.tracegen import SEED_SCALE, TraceGenerator
    lib = _abi.lib()
    N = args.objects
    K, W = args.steps, max(args.warmup, 3)
    total = W + K
    host_gen = TraceGenerator(SEED_SCALE, N)
    box = host_gen.box()
    first = host_gen.steps(1)[0]
    gen2 = TraceGenerator(SEED_SCALE, N)
    pb, ob = gen2.params_bytes(), gen2.objects_bytes()
    rt = cudart()
    rt.cudaSetDevice(local)
    step_bytes = 16 * N
    dbuf = ctypes.c_void_p()
    assert rt.cudaMalloc(ctypes.byref(dbuf), ctypes.c_size_t(step_bytes * total)) == 0
    gh = ctypes.c_void_p()
    assert lib.glint_gen_create(pb, len(pb), ob, N, len(ob) // N, 0, ctypes.byref(gh)) == 0
    for t in range(total):
        lib.glint_gen_step(gh, ctypes.c_void_p(dbuf.value + t * step_bytes), None)
    rt.cudaDeviceSynchronize()
    lib.glint_gen_destroy(gh)

    modes = ["tuned", "plain"] if args.mode == "both" else [args.mode]
    forms = {}
    for m in modes:
        forms[m] = run_form(args, m, N, local, pg, world, box, first, pb, ob, dbuf, step_bytes, rt)
    rt.cudaFree(dbuf)
    head = forms[modes[0]]
    cpu = cpu_baseline(args) if (rank == 0 and world == 1 and not args.no_cpu) else None
    if rank == 0:
        line = {"metric": METRIC, "value": head["value"], "unit": UNIT, "n_gpus": world, "steps": K, "warmup": W,
                "ms_per_step": head["ms_per_step"], "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
                "dtype": "f64", "data": "synthetic",
                "config": {"workload": f"Manhattan-grid generator (configs[1]): {N} objects, FP64 lon/lat, reach 2 m, "
                                       f"min meeting 5, leaf capacity 50, {args.buckets} buckets; headline form "
                                       f"'{modes[0]}'", "objects": N, "buckets": args.buckets, "form": modes[0],
                           "l2": "inputs larger than L2 (160 MB of points per step, 34 GB table)"},
                "roofline": roofline(head, N), "clocks": head["clocks"], "e2e": head["e2e"], "cpu_baseline": cpu,
                "gpu_launches": head["gpu_launches"],
                "forms": {m: {k: v for k, v in f.items()} for m, f in forms.items()}}
        print(json.dumps(line), flush=True)


if __name__ == "__main__":
    main()
