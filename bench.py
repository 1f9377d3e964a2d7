"""Benchmark: object-timesteps/s of the contact-tracing step at 10M objects.

Workload (BASELINE configs[1]): the seeded Manhattan-grid generator, 10M
objects, FP64 lon/lat, reach 2 m, minimum meeting 5 steps, QuadTree leaf
capacity 50 (the reference default), meeting table of 2^30 buckets.  One
step = partition -> filter -> refine -> table insert -> identify -> schema
update for one 1-second timestep of all objects.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]
                    [--objects N] [--mode plain|tuned]

value: device-resident inputs (points generated on the device beforehand),
K steps bracketed by CUDA events.  e2e: the same steps through glint_step()
with points in pinned host memory (host->device copy inside the timed region)
and each step's meetings copied back.  Under torchrun (N>1) every rank runs an
independent replica on its own GPU (the path has no data exchange), the
slowest rank's time counts and value sums all ranks' object-timesteps.
"""
from __future__ import annotations

import argparse
import ctypes
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


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=20)
    p.add_argument("--warmup", type=int, default=8)
    p.add_argument("--impl", default="glint", choices=["glint", "reference"])
    p.add_argument("--objects", type=int, default=10_000_000)
    p.add_argument("--buckets", type=int, default=1 << 30)
    p.add_argument("--mode", default="plain", choices=["plain", "tuned"])
    p.add_argument("--no-e2e", action="store_true")
    p.add_argument("--cpu-sample-objects", type=int, default=1_000_000)
    p.add_argument("--cpu-sample-steps", type=int, default=3)
    return p.parse_args()


def dist_init(gpus):
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
    """nvidia-smi sampling during the timed region."""

    def __init__(self, device):
        self.device = device
        self.proc = None
        self.path = os.path.join(ROOT, "gpurun_out", f"clocks_{os.getpid()}.csv")

    def __enter__(self):
        try:
            os.makedirs(os.path.dirname(self.path), exist_ok=True)
            q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
                 "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
                 "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), f"--query-gpu={q}",
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
        out = {"sm_mhz": None, "sm_max_mhz": None, "reasons": []}
        try:
            rows = [r.split(",") for r in open(self.path).read().strip().splitlines() if r.strip()]
        except Exception:
            return out
        sm = [float(r[1]) for r in rows if len(r) >= 9 and r[1].strip().replace(".", "").isdigit()]
        if sm:
            out["sm_mhz"] = float(np.median(sm))
            out["sm_max_mhz"] = float(rows[0][2])
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = set()
        for r in rows:
            if len(r) < 9:
                continue
            for k, name in enumerate(names):
                if "Active" in r[5 + k] and "Not" not in r[5 + k]:
                    reasons.add(name)
        out["reasons"] = sorted(reasons)
        out["samples"] = len(rows)
        return out


def peaks():
    try:
        return json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except Exception:
        return {}


def cpu_baseline(args):
    """The CPU oracle (port of the reference's stages) on a bounded sample."""
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
            "sample": f"{n} objects of the same generator (seed, box, hotspots), {k} timed steps after 1; "
                      f"single-threaded C restatement of the reference's CPU stages, -O2"}


def run_reference_arm(args, rank, world, pg):
    if rank != 0:
        return
    from glint_pipeline_gb300.tracegen import SEED_SCALE, TraceGenerator
    from oracle.bindings import Oracle, make_config
    n = args.cpu_sample_objects
    g = TraceGenerator(SEED_SCALE, n)
    box, pts = g.box(), g.steps(args.warmup + args.steps + 1)
    o = Oracle(make_config(n, num_meeting_buckets=1 << 24), box, pts[0])
    for t in range(args.warmup):
        o.step(pts[t], t)
    t0 = time.perf_counter()
    for t in range(args.warmup, args.warmup + args.steps):
        o.step(pts[t], t)
    dt = time.perf_counter() - t0
    value = n * args.steps / dt
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000 * dt / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": f"Manhattan-grid generator sample, {n} objects, reach 2 m, min meeting 5, "
                                   f"leaf capacity 50", "objects": n},
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": 1, "kind": "port",
                             "sample": f"{n} objects x {args.steps} steps per timed region (the reference's "
                                       f"sources are not on this machine; single-threaded C restatement)"},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def main():
    args = parse()
    rank, world, local, pg = dist_init(args.gpus)
    if args.impl == "reference":
        run_reference_arm(args, rank, world, pg)
        return
    import glint_pipeline_gb300 as gp
    from glint_pipeline_gb300 import _abi
    from glint_pipeline_gb300.tracegen import SEED_SCALE, TraceGenerator

    lib = _abi.lib()
    N = args.objects
    K, W = args.steps, max(args.warmup, 3)
    total = W + K
    # generator state on the host, then all steps generated on the device
    host_gen = TraceGenerator(SEED_SCALE, N)
    box = host_gen.box()
    first = host_gen.steps(1)[0]
    gen2 = TraceGenerator(SEED_SCALE, N)
    pb, ob = gen2.params_bytes(), gen2.objects_bytes()
    cfg = gp.Configuration(num_objects=N, num_meeting_buckets=args.buckets, device=local, timing=True,
                           precision_mode=1 if args.mode == "tuned" else 0)
    bench = gp.DeviceBench(cfg, box, first)
    rt = _cudart()
    # device buffer with every step's points (inputs resident in HBM)
    step_bytes = 16 * N
    dbuf = ctypes.c_void_p()
    assert rt.cudaMalloc(ctypes.byref(dbuf), ctypes.c_size_t(step_bytes * total)) == 0
    gh = ctypes.c_void_p()
    assert lib.glint_gen_create(pb, len(pb), ob, N, len(ob) // N, 0, ctypes.byref(gh)) == 0
    for t in range(total):
        lib.glint_gen_step(gh, ctypes.c_void_p(dbuf.value + t * step_bytes), ctypes.c_void_p(bench.stream))
    rt.cudaDeviceSynchronize()
    lib.glint_gen_destroy(gh)

    stage_ms = np.zeros(8)
    stats_last = None
    for t in range(W):
        bench.step_device(dbuf.value + t * step_bytes, t)
        stats_last = bench.sync()
    barrier(pg)
    contacts = candidates = meetings = new_keys = 0
    dev_ms = 0.0
    with Clocks(local) as clk:
        for t in range(W, total):
            bench.step_device(dbuf.value + t * step_bytes, t)
            st = bench.sync()  # per-step stats (tiny D2H) and per-stage CUDA-event times on the step's stream
            stage_ms += np.array(st.ms)
            dev_ms += st.ms[7]
            contacts += st.contacts
            candidates += st.candidates
            meetings += st.meetings
            new_keys += st.new_keys
            stats_last = st
    dev_s = allreduce_max(pg, dev_ms / 1000.0)
    value = N * K * world / dev_s
    clocks = clk.summary()

    # e2e: host points (pinned), copy inside the timed region, meetings copied back
    e2e = None
    if not args.no_e2e:
        ke = min(K, 8)
        hbuf = ctypes.c_void_p()
        assert rt.cudaMallocHost(ctypes.byref(hbuf), ctypes.c_size_t(step_bytes * ke)) == 0
        base = W + K
        # continue the trajectory: steps base .. base+ke-1 generated on the device, staged to host
        gh2 = ctypes.c_void_p()
        gen3 = TraceGenerator(SEED_SCALE, N)
        assert lib.glint_gen_create(gen3.params_bytes(), len(pb), gen3.objects_bytes(), N, len(ob) // N, 0,
                                    ctypes.byref(gh2)) == 0
        tmp = ctypes.c_void_p()
        rt.cudaMalloc(ctypes.byref(tmp), ctypes.c_size_t(step_bytes))
        for t in range(base + ke):
            lib.glint_gen_step(gh2, tmp, ctypes.c_void_p(bench.stream))
            if t >= base:
                rt.cudaDeviceSynchronize()
                rt.cudaMemcpy(ctypes.c_void_p(hbuf.value + (t - base) * step_bytes), tmp, ctypes.c_size_t(step_bytes),
                              2)
        rt.cudaDeviceSynchronize()
        lib.glint_gen_destroy(gh2)
        rt.cudaFree(tmp)
        arr = (ctypes.c_double * (2 * N * ke)).from_address(hbuf.value)
        host = np.frombuffer(arr, dtype=np.float64).reshape(ke, N, 2)
        barrier(pg)
        d2h = 0
        t0 = time.perf_counter()
        for k in range(ke):
            st = bench.step(host[k], base + k)
            m = bench.meetings()
            d2h += m.nbytes + ctypes.sizeof(_abi.GlintStepStats)
        dt = allreduce_max(pg, time.perf_counter() - t0)
        e2e = {"value": N * ke * world / dt, "unit": UNIT, "h2d_bytes_per_step": step_bytes,
               "d2h_bytes_per_step": int(d2h / ke), "steps": ke}
        rt.cudaFreeHost(hbuf)

    pk = peaks()
    hbm = pk.get("hbm_gbs")
    # roofline of the refine kernel (dominant): algorithmic bytes per launch =
    # 28 B per object (member tile x, y, L, id) + 32 B per candidate pair's
    # querier side is amortised in the tile; + 32 B per contact (table record
    # probe) + 1 B stamp, see the design doc
    refine_ms = stage_ms[3] / K
    refine_bytes = 28 * N + 33 * (contacts / K)
    achieved = refine_bytes / (refine_ms / 1000.0) / 1e9 if refine_ms > 0 else None
    roof = {"kernel": "k_refine_fp64", "bound": "hbm", "achieved": achieved, "peak": hbm, "unit": "GB/s",
            "frac": (achieved / hbm) if (achieved and hbm) else None, "traffic": None,
            "peak_source": "MEASURED_PEAKS.json hbm_gbs (burst copy)" if hbm else "fallback 6800"}

    cpu = cpu_baseline(args) if (rank == 0 and world == 1) else None
    if rank == 0:
        line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": K, "warmup": W,
                "ms_per_step": 1000.0 * dev_s / K, "higher_is_better": True, "scaling": "weak",
                "vs_baseline": None, "dtype": "f64", "data": "synthetic",
                "config": {"workload": f"Manhattan-grid generator (configs[1]): {N} objects, FP64 lon/lat, reach 2 m, "
                                       f"min meeting 5, leaf capacity 50, {args.buckets} buckets, {args.mode} refine",
                           "objects": N, "buckets": args.buckets, "mode": args.mode,
                           "l2": "inputs larger than L2 (160 MB points per step, 34 GB table)"},
                "stage_ms": {k: v / K for k, v in zip(["copy", "partition", "filter", "refine", "insert", "identify",
                                                      "schema", "total"], stage_ms)},
                "per_step": {"candidates": candidates / K, "contacts": contacts / K, "new_keys": new_keys / K,
                             "meetings": meetings / K, "checks": stats_last.checks, "leaves": stats_last.leaves,
                             "ambiguous": stats_last.ambiguous, "rechecks": stats_last.rechecks,
                             "error_flags": stats_last.error_flags},
                "roofline": roof, "clocks": clocks, "e2e": e2e, "cpu_baseline": cpu,
                "gpu_launches": None}
        print(json.dumps(line), flush=True)
    bench.close()
    rt.cudaFree(dbuf)


def _cudart():
    import glob
    for cand in ["libcudart.so", "libcudart.so.13"] + glob.glob("/usr/local/cuda/lib64/libcudart.so*"):
        try:
            lib = ctypes.CDLL(cand)
            lib.cudaEventElapsedTime.argtypes = [ctypes.POINTER(ctypes.c_float), ctypes.c_void_p, ctypes.c_void_p]
            lib.cudaEventRecord.argtypes = [ctypes.c_void_p, ctypes.c_void_p]
            lib.cudaEventSynchronize.argtypes = [ctypes.c_void_p]
            lib.cudaMemcpy.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t, ctypes.c_int]
            lib.cudaFree.argtypes = [ctypes.c_void_p]
            lib.cudaFreeHost.argtypes = [ctypes.c_void_p]
            return lib
        except OSError:
            continue
    raise OSError("libcudart not found")


if __name__ == "__main__":
    main()
