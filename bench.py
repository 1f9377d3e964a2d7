"""Benchmark: object-timesteps/s of the contact-tracing step at 10M objects.

Workload: the seeded Manhattan-grid generator (40x40 km, 8 hotspots), 10M
objects, FP64 lon/lat, reach 2 m, minimum meeting 5 steps, QuadTree leaf
capacity 50 (the reference default), a meeting table of 2^30 buckets.  One
step = partition -> filter -> refine -> table insert -> identify (+ keys) ->
schema update for one 1-second timestep of all objects, plus the flush into
the key-value store whenever more than kv_restriction keys are pending (as
the reference's loop does).  Both forms produce bit-identical meetings;
"plain" runs the reference's FP64 test on every candidate pair, "tuned"
screens pairs in FP32 with a guard band first.  After the steps, the serving
form answers a Poisson stream of contact-trace queries against the flushed
store (p50/p99 latency, queries/s), and the compaction leg merges the kept
blocks into one of 56^2 CTFs (merge_dump), with a 500k-object sample merged
by the device and by the oracle on the host and compared bit for bit.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]
                    [--objects N] [--mode both|plain|tuned]

value: device-resident inputs (every step's points generated on the device
beforehand), the K timed steps measured with CUDA events on the step's
stream.  e2e: further steps through the pipelined API (glint_pipe_*) with
points in pinned host memory (host->device copy inside the timed region,
overlapped with the step before) and each step's meetings read back from
page-locked result buffers.  Under torchrun (N>1) every rank runs an independent replica on
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
    p.add_argument("--e2e-steps", type=int, default=20,
                   help="host-buffer steps timed through the pipelined API (as many as the timed steps, so the "
                        "flushes amortise alike)")
    p.add_argument("--no-e2e", action="store_true", help="skip the host-buffer pass (profiling runs)")
    p.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline (profiling runs)")
    p.add_argument("--cpu-steps", type=int, default=11,
                   help="steps the oracle times on the headline workload after --cpu-warmup (its meetings are "
                        "compared with the GPU's on all of them)")
    p.add_argument("--cpu-warmup", type=int, default=1)
    p.add_argument("--cpu-threads", type=int, default=0, help="0: all host cores")
    p.add_argument("--serve-seconds", type=float, default=6.0,
                   help="Poisson stream length; 0 serves only the 2-hop queries from 1000 seeds")
    p.add_argument("--serve-rate", type=float, default=200.0)
    p.add_argument("--serve-sweep", default="50,2000",
                   help="further Poisson rates (req/s) served for --serve-seconds / 2 each; empty: none")
    p.add_argument("--no-serve", action="store_true")
    p.add_argument("--serve-deadline", type=float, default=20.0,
                   help="seconds after a stream's last arrival before its unfinished queries are given up")
    p.add_argument("--serve-reserve-gb", type=float, default=8.0,
                   help="device memory left free for the query slots when the store moves onto the device")
    p.add_argument("--serve-steps", type=int, default=1800,
                   help="steps of the serving store's build (the serving configuration: 10M objects x 1800 s)")
    p.add_argument("--serve-device-gb", type=float, default=230.0, help="device memory for kept store blocks")
    p.add_argument("--serve-host-gb", type=float, default=90.0,
                   help="page-locked host memory for the kept store blocks before the device's")
    p.add_argument("--compact-split", type=int, default=56,
                   help="split_num of the compaction leg (the reference tool merges into 56^2 = 3136 CTFs)")
    p.add_argument("--compact-sample-objects", type=int, default=500_000)
    p.add_argument("--no-compact", action="store_true")
    p.add_argument("--workload", default="step10m", choices=["step10m", "batch64", "skew50m", "compact", "serve"],
                   help="step10m: the headline line; batch64 / skew50m: the batching and precision forms; "
                        "compact: the compaction sample alone (--compact-sample-objects objects); serve: the "
                        "serving leg alone (store build over --serve-steps, then the queries)")
    p.add_argument("--serve-kv", type=int, default=0,
                   help="keys pending before the serving store's build flushes a block; 0: the default 2^26")
    p.add_argument("--regions", type=int, default=64)
    p.add_argument("--form-steps", type=int, default=6,
                   help="timed steps of the batching and skew legs inside the default run (their own "
                        "--workload runs use --steps)")
    p.add_argument("--no-forms", action="store_true", help="skip the batching and skew legs of the default run")
    p.add_argument("--skew-objects", type=int, default=50_000_000)
    p.add_argument("--skew-buckets", type=int, default=1 << 31)
    p.add_argument("--core-objects", type=int, default=2_000_000)
    p.add_argument("--core-buckets", type=int, default=0, help="0: 256 per object, rounded up to a power of two")
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
        import tempfile
        fd, self.path = tempfile.mkstemp(prefix=f"glint_clocks_{tag}_", suffix=".csv")
        os.close(fd)

    def __enter__(self):
        try:
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
        finally:
            try:
                os.unlink(self.path)
            except OSError:
                pass
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
    """Algorithmic bytes of one step of a stage: per-unit figures x units."""
    if stage == "refine":
        # member tile (X, Y, cx, f32 x/y, id: 32 B/object); per cross check the
        # check and the querier's record (48 B); per contact the table record
        # read (32 B), its box written (16 B) and its stamp (1 B); per new pair
        # a 16-B new-list entry
        return 32 * N + 48 * st["cross_checks"] + 49 * st["contacts"] + 16 * st["new_keys"]
    if stage == "identify":
        # stamps (2 B/bucket over two passes); per expiring entry its record
        # read and reset (48 B); per new entry its finalisation (80 B); per
        # reported meeting the record, log entry and two keys with boxes (128 B)
        return 2 * st["buckets"] + 48 * st["expired"] + 80 * st["new_keys"] + 128 * st["meetings"]
    if stage == "filter":
        # per object its leaf words and counts (24 B); per border object its
        # coordinates and scale (36 B); per check 24 B over the two lists
        return 24 * N + 36 * st["border_objects"] + 24 * st["cross_checks"]
    if stage == "insert":
        # per new pair: list entry (16 B), record compare-and-swap read and
        # write (64 B); the line bitmap it marks stays in L2
        return 80 * st["new_keys"]
    if stage == "partition":
        # point and order reads, three leaf words, scatter, segment sort, and
        # the gather of six per-object arrays
        return 124 * N
    return 0


def run_form(args, mode, N, local, pg, world, box, first, pb, ob, dbuf, step_bytes, rt):
    import glint_pipeline_gb300 as gp
    from glint_pipeline_gb300 import _abi
    from glint_pipeline_gb300.tracegen import SEED_SCALE, TraceGenerator
    lib = _abi.lib()
    K, W = args.steps, max(args.warmup, 3)
    cfg = gp.Configuration(num_objects=N, num_meeting_buckets=args.buckets, device=local, timing=True,
                           precision_mode=1 if mode == "tuned" else 0, auto_flush=True)
    bench = gp.DeviceBench(cfg, box, first)
    digests = MeetingDigests(N)
    for t in range(W):
        bench.step_device(dbuf.value + t * step_bytes, t)
        bench.sync()
        digests.add(bench)
    barrier(pg)
    stage_ms = np.zeros(8)
    flush_ms, flushes = 0.0, 0
    acc = {"candidates": 0, "contacts": 0, "new_keys": 0, "meetings": 0, "cross_checks": 0, "border_objects": 0,
           "taken": 0, "active": 0, "band_pairs": 0, "box_band": 0, "rechecks": 0, "ambiguous": 0}
    launches = 0
    dev_ms = 0.0
    last = None
    with Clocks(local, mode) as clk:
        for t in range(W, W + K):
            bench.step_device(dbuf.value + t * step_bytes, t)
            st = bench.sync()
            digests.add(bench)
            stage_ms += np.array(st.ms)
            dev_ms += st.ms[7] + st.flush_ms
            flush_ms += st.flush_ms
            flushes += int(st.flushed)
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
            acc["box_band"] += st.box_band
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
    stage = {k: v / K for k, v in zip(STAGES, stage_ms)}
    stage["flush"] = flush_ms / K
    stage["total"] = stage["total"] + stage["flush"]
    per["flushes"] = flushes
    out = {"value": N * K * world / dev_s, "ms_per_step": 1000.0 * dev_s / K,
           "stage_ms": stage, "per_step": per,
           "clocks": clk.summary(), "gpu_launches": launches}
    out["_digests"], out["_meetings"] = digests.result()

    if args.no_e2e:
        out["e2e"] = None
        out["_bench"] = bench
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
    # pipelined stepping (glint_pipe_*): step k+1's points are copied from
    # page-locked memory while step k computes, and each step's meetings are
    # written into page-locked result buffers and read here
    pipe = gp.Pipe(bench, result_capacity=N)
    barrier(pg)
    d2h = 0
    t0 = time.perf_counter()
    pipe.submit(host[0], base)
    for k in range(ke):
        if k + 1 < ke:
            pipe.submit(host[k + 1], base + k + 1)
        st_k, m = pipe.result(base + k)
        d2h += m.nbytes + ctypes.sizeof(_abi.GlintStepStats)
    dt = allreduce_max(pg, time.perf_counter() - t0)
    del m
    pipe.close()
    out["e2e"] = {"value": N * ke * world / dt, "unit": UNIT, "h2d_bytes_per_step": step_bytes,
                  "d2h_bytes_per_step": int(d2h / ke), "steps": ke}
    del host, arr
    rt.cudaFreeHost(hbuf)
    out["_bench"] = bench
    return out


# DRAM bytes per step of each stage's kernels (dram__bytes_read.sum +
# dram__bytes_write.sum) at 10M objects and 2^30 buckets, the tuned form:
# from a full capture of each kernel on the 2M-object case scaled by the
# stage's units, and from the one-pass launch list of the 10M step where
# noted (profiles/); other workloads report null
TRAFFIC_10M_2P30 = {"refine": 43.0e9, "identify": 50.6e9, "insert": 26.5e9}


def step_bytes_8d(N, per):
    """Algorithmic bytes of one step by the hot path's byte model:
    40 B per object (16 B of coordinates read, 4 B leaf key and 4 B id
    written, 16 B of coordinates re-read in leaf order), 32 B per contact
    pair (its 16-B table entry read and written) and 48 B per completed
    meeting (the 16-B record and two 16-B keys); split by stage as the
    kernels move them."""
    by = {"partition": 24 * N, "filter": 0, "refine": 16 * N + 32 * per["contacts"], "insert": 0,
          "identify": 48 * per["meetings"]}
    return 40 * N + 32 * per["contacts"] + 48 * per["meetings"], by


def roofline(form, N, buckets=None, mode=None):
    pk = peaks()
    hbm = pk.get("hbm_gbs")
    peak = hbm if hbm else 6800.0
    stages = {k: v for k, v in form["stage_ms"].items() if k in ("partition", "filter", "refine", "insert", "identify")}
    # the dominant kernel is refine's (k_refine_fp32 in the tuned form: 35% of
    # the step's kernel time in the ncu launch list, k_expire_count next at
    # 26%); by stage, refine and identify take turns as the slowest
    top = "refine"
    slowest = max(stages, key=stages.get)
    ms = stages[top]
    step_by, by8 = step_bytes_8d(N, form["per_step"])
    by = by8[top]
    achieved = by / (ms / 1000.0) / 1e9 if ms > 0 else None
    measured = N == 10_000_000 and buckets == 1 << 30 and mode == "tuned"
    traffic = TRAFFIC_10M_2P30.get(top) if measured else None
    stage_model = {k: stage_bytes(k, N, form["per_step"], 1) for k in stages}
    ratio = {k: (TRAFFIC_10M_2P30[k] / by8[k] if by8.get(k) else None) for k in TRAFFIC_10M_2P30} if measured else None
    kernel = "k_refine_fp32" if mode == "tuned" else "k_refine_fp64"
    return {"kernel": kernel, "kernel_stage": top, "slowest_stage": slowest, "bound": "hbm", "achieved": achieved,
            "peak": peak, "unit": "GB/s",
            "frac": achieved / peak if achieved else None, "traffic": traffic,
            "traffic_unit": "DRAM bytes per step of the stage's kernels", "algorithmic_bytes": by,
            "model": "40 B/object + 32 B/contact pair + 48 B/meeting; the stage's share",
            "step_bytes": step_by, "frac_step": step_by / (form["ms_per_step"] / 1000.0) / 1e9 / peak,
            # the model's flush term: 2 x 16 B per key and radix pass over the
            # flushed keys (two per reported meeting), 16 passes of 8 bits for
            # 128-bit keys, amortised over the steps
            "flush_bytes_per_step": 2 * 16 * 16 * 2 * form["per_step"]["meetings"],
            "frac_step_with_flush": (step_by + 2 * 16 * 16 * 2 * form["per_step"]["meetings"]) /
                                    (form["ms_per_step"] / 1000.0) / 1e9 / peak,
            "traffic_over_algorithmic": ratio,
            "stage_model_bytes": stage_model,
            "stage_model": "bytes each stage's kernels must move in this design (table records, lists, "
                           "stamps); the `model` above counts only 40 B/object, 32 B/contact and 48 B/meeting",
            "peak_source": "of measured (MEASURED_PEAKS.json hbm_gbs)" if hbm else "of fallback"}


def host_memory_available():
    """Bytes this process may still allocate: MemAvailable, capped by a
    cgroup limit where one is set."""
    avail = None
    try:
        for line in open("/proc/meminfo"):
            if line.startswith("MemAvailable:"):
                avail = int(line.split()[1]) * 1024
    except OSError:
        pass
    for path, used_path in (("/sys/fs/cgroup/memory.max", "/sys/fs/cgroup/memory.current"),
                            ("/sys/fs/cgroup/memory/memory.limit_in_bytes",
                             "/sys/fs/cgroup/memory/memory.usage_in_bytes")):
        try:
            lim = open(path).read().strip()
            if lim != "max" and int(lim) < (1 << 60):
                room = int(lim) - int(open(used_path).read().strip())
                avail = room if avail is None else min(avail, room)
            break
        except (OSError, ValueError):
            continue
    return avail


def oracle_bytes(N, B):
    """host memory the oracle needs at N objects and B buckets: the table,
    the leaf buffers and their coordinates, the meeting list and the
    per-step contact lists"""
    grids = 4 * max(100_000, N // 50)
    return 32 * B + grids * 100 * 20 + 1100 * N


def cpu_baseline(args, N, B, steps, warm, gpu_digests=None):
    """The reference's CPU stages, as the oracle's C restatement (-O2), on
    the host cores and on the GPU arm's own workload: the generator at N
    objects from step 0, B buckets, leaf capacity 50.  The restatement runs
    the order-free parts on all host threads and gives the results of one
    thread.  Timed: steps warm .. warm+steps-1 (wall clock around each
    step).  Every step's meetings are digested as the GPU's are; with
    gpu_digests given, they are compared step by step."""
    from glint_pipeline_gb300 import MEETING_DTYPE
    from glint_pipeline_gb300.tracegen import SEED_SCALE, TraceGenerator
    from oracle.bindings import Oracle, cantor_inverse, make_config
    threads = args.cpu_threads or os.cpu_count() or 1
    need, avail = oracle_bytes(N, B) + 16 * N * (warm + steps), host_memory_available()
    if avail is not None and need > 0.8 * avail:
        return {"skipped": f"the oracle needs about {need / 1e9:.0f} GB of host memory; {avail / 1e9:.0f} GB "
                           f"available"}
    total = warm + steps
    g = TraceGenerator(SEED_SCALE, N)
    box, pts = g.box(), g.steps(total)
    g.close()
    t0 = time.perf_counter()
    o = Oracle(make_config(N, num_meeting_buckets=B), box, pts[0], threads=threads)
    create_s = time.perf_counter() - t0
    step_s, digests, counts = [], [], []
    try:
        for t in range(total):
            t0 = time.perf_counter()
            o.step(pts[t], t)
            dt = time.perf_counter() - t0
            if t >= warm:
                step_s.append(dt)
            mo = o.meetings()
            rec = np.zeros(mo.shape[0], MEETING_DTYPE)
            rec["pid1"], rec["pid2"] = cantor_inverse(mo["key"])
            rec["start"], rec["end"], rec["mbr"] = mo["start"], mo["end"], mo["mbr"]
            digests.append(meeting_digest(rec))
            counts.append(int(rec.shape[0]))
            del mo, rec
    finally:
        o.close()
    wall = float(sum(step_s))
    out = {"value": N * steps / wall, "unit": UNIT, "cores": threads, "kind": "port",
           "sample": f"the GPU arm's workload itself ({N} objects, {B} buckets), steps {warm}..{total - 1} "
                     f"timed after {warm} untimed; the reference's CPU stages as the C restatement, "
                     f"{threads} host threads (results identical to one thread)",
           "ms_per_step": 1000.0 * wall / steps, "steps": steps, "warmup": warm, "create_s": create_s,
           "cpu_model": cpu_model(), "host_threads_available": os.cpu_count(), "same_config": True}
    if gpu_digests is not None:
        n = min(len(gpu_digests), len(digests))
        diff = [t for t in range(n) if gpu_digests[t] != digests[t]]
        out["parity"] = {"steps": n, "meetings": int(sum(counts[:n])),
                         "steps_with_meetings": int(sum(1 for c in counts[:n] if c)), "mismatching_steps": diff,
                         "compared": "every step's meetings (pid1, pid2, start, end, f32 box bits) in bucket order, "
                                     "tuned GPU form vs the oracle, SHA-256"}
    return out


def cpu_model():
    """The host CPU's model name (/proc/cpuinfo; Arm hosts give an implementer
    and part number instead)."""
    try:
        info = open("/proc/cpuinfo").read()
    except OSError:
        return None
    for key in ("model name", "Model", "Hardware"):
        for line in info.splitlines():
            if line.startswith(key) and ":" in line:
                return line.split(":", 1)[1].strip()
    impl = part = None
    for line in info.splitlines():
        if line.startswith("CPU implementer"):
            impl = line.split(":", 1)[1].strip()
        if line.startswith("CPU part"):
            part = line.split(":", 1)[1].strip()
    parts = {"0xd4f": "Arm Neoverse V2", "0xd40": "Arm Neoverse V1", "0xd0c": "Arm Neoverse N1"}
    if part:
        return f"{parts.get(part, 'Arm part ' + part)} (implementer {impl})"
    return None


def run_reference_arm(args, rank, world, pg):
    if rank != 0:
        return
    steps = max(1, min(args.steps, 3))
    warm = max(1, min(args.warmup, 2))
    N, B = args.objects, args.buckets
    cb = cpu_baseline(args, N, B, steps, warm)
    if "skipped" in cb:
        print(json.dumps({"impl": "reference", "unavailable": cb["skipped"]}), flush=True)
        return
    value = cb["value"]
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
            "steps": steps, "warmup": warm, "ms_per_step": cb["ms_per_step"], "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": workload_config(args, N, "reference CPU stages (C restatement)"),
            "cpu_baseline": {k: cb[k] for k in ("value", "unit", "cores", "kind", "sample", "cpu_model",
                                                "same_config")},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def workload_config(args, N, form):
    return {"workload": f"Manhattan-grid generator (40x40 km, 8 hotspots): {N} objects, FP64 lon/lat, reach 2 m, "
                        f"min meeting 5, leaf capacity 50, {args.buckets} buckets, flush past 2^26 keys; "
                        f"headline form '{form}'",
            "objects": N, "buckets": args.buckets, "form": form,
            "l2": (f"inputs larger than L2 ({16 * N / 1e6:.0f} MB of points per step, "
                   f"{32 * args.buckets / 1e9:.1f} GB table)" if 32 * args.buckets > 129e6 else
                   f"the table ({32 * args.buckets / 1e6:.0f} MB) fits in L2")}


def poisson_stream(srv, rng, N, t_hi, rate, seconds, deadline_s):
    """queries arriving at `rate` for `seconds`, each submitted when it
    arrives and retired when its last hop is done; those not done
    `deadline_s` after the last arrival are left unfinished (counted, not
    waited for).  Returns latencies of the finished queries (ms), wall time,
    objects reached, queries, unfinished"""
    n = max(1, int(rate * seconds))
    arrive = np.cumsum(rng.exponential(1.0 / rate, n))
    qs = []
    for _ in range(n):
        k = int(np.exp(rng.uniform(0, np.log(1000))))
        hops = int(rng.integers(1, 4))
        length = float(np.exp(rng.uniform(np.log(10), np.log(1800))))
        t0 = int(rng.integers(0, max(1, t_hi)))
        qs.append((rng.choice(N, k, replace=False).astype(np.uint32), hops, t0, t0 + int(length)))
    lat, inflight, i = [], {}, 0
    reached = 0
    t_start = time.perf_counter()
    stop_at = arrive[-1] + deadline_s
    while len(lat) < n:
        now = time.perf_counter() - t_start
        if now > stop_at:
            break
        while i < n and arrive[i] <= now:
            inflight[srv.submit(*qs[i])] = arrive[i]
            i += 1
        if not inflight:
            time.sleep(max(0.0, arrive[i] - now))
            continue
        srv.step()
        done_t = time.perf_counter() - t_start
        for tk in list(inflight):
            r = srv.poll(tk, cap=1)
            if r is not None:
                lat.append(done_t - inflight.pop(tk))
                reached += r[2]
    wall = time.perf_counter() - t_start
    unfinished = n - len(lat)
    # a server is not reused after a stream that left queries behind
    return np.array(lat) * 1000.0, wall, reached, n, unfinished


def latency_summary(lat, n, unfinished, deadline_s):
    """p50/p99 over all arrivals: unfinished queries count as slower than any
    finished one (p99 is null when more than 1% did not finish by the
    deadline)"""
    out = {"queries": n, "finished": n - unfinished, "deadline_s": deadline_s}
    if unfinished == 0:
        out.update({"p50_ms": float(np.percentile(lat, 50)), "p99_ms": float(np.percentile(lat, 99))})
        return out
    srt = np.sort(lat)
    for p in (50, 99):  # nearest rank over all arrivals; null past the finished ones
        k = int(np.ceil(p / 100.0 * n)) - 1
        out[f"p{p}_ms"] = float(srt[k]) if k < len(srt) else None
    return out


def serving(args, bench, N, t_hi, sweep_rates=True):
    """Poisson stream of contact-trace queries against the flushed store,
    served with continuous batching, at --serve-rate and the --serve-sweep
    rates; plus 2-hop queries from 1000 seeds alone."""
    import glint_pipeline_gb300 as gp
    if bench.store_blocks() == 0:
        return None
    rng = np.random.default_rng(0x474C494E54000005)
    dl = args.serve_deadline
    srv = gp.Server(bench, max_slots=64)
    if args.serve_seconds > 0:
        lat, wall, reached, n, unf = poisson_stream(srv, rng, N, t_hi, args.serve_rate, args.serve_seconds, dl)
        main = latency_summary(lat, n, unf, dl)
    else:
        wall, reached, n, unf, main = 1.0, 0, 0, 0, {}
        sweep_rates = False
    sweep = {}
    rates = [float(x) for x in args.serve_sweep.split(",") if x.strip() and sweep_rates]
    left = unf
    for r in rates:
        if left:
            srv.close()
            srv = gp.Server(bench, max_slots=64)
        sl, sw, _, sn, su = poisson_stream(srv, rng, N, t_hi, r, args.serve_seconds / 2, dl)
        sweep[f"{r:g}"] = dict(latency_summary(sl, sn, su, dl), qps=(sn - su) / sw)
        left = su
    if left:
        srv.close()
        srv = gp.Server(bench, max_slots=64)
    # 2-hop queries from 1000 seeds, one at a time, within --serve-deadline in total
    two, two_reached = [], []
    t_all = time.perf_counter()
    for _ in range(20):
        if time.perf_counter() - t_all > dl:
            break
        seeds = rng.choice(N, 1000, replace=False).astype(np.uint32)
        t0 = time.perf_counter()
        tk = srv.submit(seeds, 2)
        r = None
        while r is None:
            srv.step()
            r = srv.poll(tk, cap=1)
        two.append((time.perf_counter() - t0) * 1000.0)
        two_reached.append(r[2])
    srv.close()
    two = np.array(two)
    res = dict(main, rate_req_s=args.serve_rate, qps=(n - unf) / wall, slots=srv.slots,
               store_blocks=bench.store_blocks(), mean_reached=reached / max(1, n - unf), rates=sweep,
               mix="seeds 1-1000 log-uniform, 1-3 hops, window 10-1800 s log-uniform")
    res["two_hop_1k_seeds"] = {"p50_ms": float(np.percentile(two, 50)) if len(two) else None,
                               "p99_ms": float(np.percentile(two, 99)) if len(two) else None,
                               "queries": len(two), "mean_reached": float(np.mean(two_reached)) if two_reached else None}
    return res


def serving_store(args, local, N, pb, ob, box, first):
    """The serving configuration: a store built on the device from N objects
    over --serve-steps steps of the same generator (auto flush past 2^26
    keys), then the Poisson query stream against it.  The whole store does
    not fit one GPU beside the meeting table (about 12.4M keys, 190 MB
    packed, per step at 10M objects), so the most recent blocks stay on the
    device and the ones before them in page-locked host memory, as far as
    the --serve-device-gb / --serve-host-gb budgets go; older blocks are
    dropped.  The line says how much of the history is served."""
    import glint_pipeline_gb300 as gp
    from glint_pipeline_gb300 import _abi
    lib = _abi.lib()
    rt = cudart()
    rt.cudaSetDevice(local)
    steps = args.serve_steps
    free, total = ctypes.c_size_t(), ctypes.c_size_t()
    rt.cudaMemGetInfo(ctypes.byref(free), ctypes.byref(total))
    # a kept block: the packed keys of one window (2^26 keys plus one step's
    # overshoot, about 15 bytes each) and 10 bytes per object of indexes
    block_bytes = ((1 << 26) + 6_000_000) * 15 + 10 * N
    ctx_bytes = 32 * args.buckets + 700 * N
    dev_budget = min(args.serve_device_gb * 1e9, free.value - ctx_bytes - 20e9)
    avail = host_memory_available() or 0
    host_budget = min(args.serve_host_gb * 1e9, 0.45 * avail)
    keep = max(1, int(dev_budget // block_bytes))
    host_keep = max(0, int(host_budget // block_bytes))
    cfg = gp.Configuration(num_objects=N, num_meeting_buckets=args.buckets, device=local, precision_mode=1,
                           auto_flush=True, store_keep=keep, store_host_keep=host_keep,
                           kv_restriction=args.serve_kv)
    bench = gp.DeviceBench(cfg, box, first)
    gh = ctypes.c_void_p()
    assert lib.glint_gen_create(pb, len(pb), ob, N, len(ob) // N, 0, ctypes.byref(gh)) == 0
    buf = ctypes.c_void_p()
    assert rt.cudaMalloc(ctypes.byref(buf), ctypes.c_size_t(16 * N)) == 0
    flushes, keys_total = 0, 0
    t0 = time.perf_counter()
    try:
        for t in range(steps):
            lib.glint_gen_step(gh, buf, ctypes.c_void_p(bench.stream))
            bench.step_device(buf.value, t)
            st = bench.sync()
            if st.error_flags:
                raise RuntimeError(f"serving store build: step {t} error flags {st.error_flags:#x}")
            if st.flushed:
                flushes += 1
                last = bench.block_info(bench.store_blocks() - 1).store
                keys_total += int(last.kv_count) + int(last.oversize_kv_count)
        build_s = time.perf_counter() - t0
        lib.glint_gen_destroy(gh)
        gh = None
        rt.cudaFree(buf)
        buf = None
        # serving needs no meeting table: release the step state and bring
        # the host-kept blocks onto the device
        on_device = bench.serve_only(reserve=int(args.serve_reserve_gb * 1e9))
        nb = bench.store_blocks()
        infos = [bench.block_info(i).store for i in range(nb)]
        kept_keys = sum(int(i.kv_count) + int(i.oversize_kv_count) for i in infos)
        res = serving(args, bench, N, steps)
        res["store"] = {"objects": N, "steps_built": steps, "build_s": build_s, "flushes": flushes,
                        "blocks_kept": nb, "blocks_on_device_while_stepping": min(nb, keep),
                        "blocks_on_device_serving": on_device, "blocks_in_host_memory_serving": nb - on_device,
                        "keys_flushed": keys_total,
                        "keys_kept": kept_keys,
                        "history_fraction_kept": kept_keys / keys_total if keys_total else None,
                        "steps_kept_from": min(int(i.end_time_min) for i in infos) if infos else None,
                        "budgets_gb": {"device": dev_budget / 1e9, "host": host_budget / 1e9},
                        "note": "while stepping the newest blocks stay on the device and the ones before them "
                                "in page-locked host memory (older ones would be dropped); for serving the "
                                "meeting table is released and host-kept blocks move onto the device"}
        return res
    finally:
        if gh:
            lib.glint_gen_destroy(gh)
        if buf:
            rt.cudaFree(buf)
        bench.close()


def compaction(args, bench):
    """merge_dump at full scale: every kept block of the timed run merged into
    one block of split_num^2 CTFs on the device (glint_store_compact)."""
    nb = bench.store_blocks()
    if nb < 2:
        return None
    infos = [bench.block_info(i).store for i in range(nb)]
    src_keys = sum(int(i.kv_count) for i in infos)
    src_bytes = sum(int(i.key_bytes) for i in infos)
    t0 = time.perf_counter()
    try:
        info = bench.compact(0, nb, args.compact_split)
    except Exception as e:  # a domain error of the reference's merge is reported, not fatal
        return {"blocks": nb, "split_num": args.compact_split, "error": str(e)}
    wall = (time.perf_counter() - t0) * 1000.0
    ms = info["ms"]
    # the merged block merged again: the same keys, with the context's
    # compaction memory already mapped
    again = bench.compact(0, 1, args.compact_split)
    return {"blocks": nb, "split_num": args.compact_split, "ctfs": info["CTF_count"], "source_keys": src_keys,
            "again_ms": again["ms"], "again_source_keys_per_s": info["kv_count"] / (again["ms"] / 1000.0),
            "keys": info["kv_count"], "oversize_keys": info["oversize_kv_count"], "padding": info["padding"],
            "placed_objects": info["sid_count"], "ms": ms, "wall_ms": wall,
            "source_keys_per_s": src_keys / (ms / 1000.0),
            "packed_GBps": (src_bytes + info["key_bytes"]) / (ms / 1000.0) / 1e9,
            "note": "ms: CUDA events around the merge on the context's stream (host steps between its launches "
                    "included; first use of the context's compaction memory); again_ms: the merged block merged "
                    "once more (memory mapped); packed_GBps: source and merged packed key bytes over ms"}


def compaction_sample(args, local):
    """The same merge on a sample the host can check: the generator at
    --compact-sample-objects objects, three flushed windows, all blocks merged
    on the device and by the oracle's C restatement (one thread), whose
    results must be equal bit for bit.  A flush every 12 steps: earlier
    windows leave CTFs without keys, outside the reference's flush domain."""
    import glint_pipeline_gb300 as gp
    from glint_pipeline_gb300.tracegen import SEED_SCALE, TraceGenerator
    from oracle.bindings import compact_blocks
    n = args.compact_sample_objects
    if n <= 0:
        return None
    steps = 36
    g = TraceGenerator(SEED_SCALE + 0x5a5a, n)
    box, pts = g.box(), g.steps(steps)
    cfg = gp.Configuration(num_objects=n, num_meeting_buckets=next_pow2(64 * n), device=local, store_keep=16)
    b = gp.DeviceBench(cfg, box, pts[0])
    try:
        for t in range(steps):
            b.step(pts[t], t)
            if t % 12 == 11:
                b.flush()
        nb = b.store_blocks()
        blocks = [b.block(i) for i in range(nb)]
        src_keys = sum(int(x["ctfs"]["CTF_kv_capacity"].sum()) for x in blocks)
        split = max(2, min(args.compact_split, int(round((n / 60.0) ** (1.0 / 3.0)))))
        t0 = time.perf_counter()
        rc, want = compact_blocks(blocks, n, box, split)
        cpu_s = time.perf_counter() - t0
        if rc != 0:
            return {"objects": n, "blocks": nb, "split_num": split, "error": f"oracle rc {rc}"}
        info = b.compact(0, nb, split)
        got = b.block(0)
        equal = rc == 0 and all(np.array_equal(got[k], want[k]) for k in ("sids", "keys", "bitmaps", "o_keys"))
        equal = equal and np.array_equal(got["ctfs"].view(np.uint8), want["ctfs"].view(np.uint8))
        return {"objects": n, "blocks": nb, "split_num": split, "source_keys": src_keys, "gpu_ms": info["ms"],
                "cpu_ms": cpu_s * 1000.0, "cpu": "oracle C restatement, 1 thread", "bit_exact": bool(equal),
                "gpu_source_keys_per_s": src_keys / (info["ms"] / 1000.0), "cpu_source_keys_per_s": src_keys / cpu_s}
    finally:
        b.close()


def next_pow2(v):
    p = 1
    while p < v:
        p <<= 1
    return p


def run_batch(args, local, K=None, W=None):
    """Batching form: R regions, populations log-uniform in [1k, 2M], each with
    its own generator seed, street grid and hotspots, advanced together
    (glint_batch_*: one graph per timestep, one refine launch over all
    regions) against the same regions stepped one after another without
    graphs; an autotuner picks leaf capacity, hash load factor and refine tile
    width per size class for a tuned run."""
    import glint_pipeline_gb300 as gp
    from glint_pipeline_gb300 import _abi
    from glint_pipeline_gb300.batch import Batch, autotune
    from glint_pipeline_gb300.tracegen import SEED_REGIONS, TraceGenerator
    lib = _abi.lib()
    rt = cudart()
    rt.cudaSetDevice(local)
    R = args.regions
    rng = np.random.default_rng(SEED_REGIONS)
    pops = np.exp(rng.uniform(np.log(1_000), np.log(2_000_000), R)).astype(np.int64)
    K = args.steps if K is None else K
    W = max(args.warmup if W is None else W, 3)
    total = W + K
    regions = []
    for r in range(R):
        n = int(pops[r])
        ext = float(np.clip(40000.0 * np.sqrt(n / 10_000_000), 2000.0, 40000.0))
        g = TraceGenerator(SEED_REGIONS ^ (r + 1), n, 0, extent_m=ext)
        g2 = TraceGenerator(SEED_REGIONS ^ (r + 1), n, 0, extent_m=ext)
        box, first = g.box(), g.steps(1)[0]
        pb, ob = g2.params_bytes(), g2.objects_bytes()
        buf = ctypes.c_void_p()
        assert rt.cudaMalloc(ctypes.byref(buf), ctypes.c_size_t(16 * n * total)) == 0
        gh = ctypes.c_void_p()
        assert lib.glint_gen_create(pb, len(pb), ob, n, len(ob) // n, 0, ctypes.byref(gh)) == 0
        for t in range(total):
            lib.glint_gen_step(gh, ctypes.c_void_p(buf.value + 16 * n * t), None)
        rt.cudaDeviceSynchronize()
        lib.glint_gen_destroy(gh)
        inp = ctypes.c_void_p()
        assert rt.cudaMalloc(ctypes.byref(inp), ctypes.c_size_t(16 * n)) == 0
        regions.append({"n": n, "box": box, "first": first, "steps": buf, "input": inp})

    def config(n, cap=50, lf=None, chunk=0):
        b = next_pow2(int(64 * n)) if lf is None else next_pow2(int(28 * n / lf))
        return gp.Configuration(num_objects=n, num_meeting_buckets=b, grid_capacity=cap, precision_mode=1,
                                auto_flush=True, kv_restriction=max(1 << 20, 8 * n), store_keep=2, device=local,
                                refine_chunk=chunk)

    def copy_in(t, streams):
        for r, reg in enumerate(regions):
            rt.cudaMemcpyAsync(reg["input"], ctypes.c_void_p(reg["steps"].value + 16 * reg["n"] * t),
                               ctypes.c_size_t(16 * reg["n"]), 3, ctypes.c_void_p(streams[r]))

    def batched(cfgs):
        batch = Batch(cfgs, [x["box"] for x in regions], [x["first"] for x in regions])
        streams = [batch.stream(r) for r in range(R)]
        ptrs = [x["input"].value for x in regions]
        for t in range(W):
            copy_in(t, streams)
            batch.step(ptrs, t)
            batch.sync()
        rt.cudaDeviceSynchronize()
        with Clocks(local, "batch") as clk:
            t0 = time.perf_counter()
            for t in range(W, total):
                copy_in(t, streams)
                batch.step(ptrs, t)
                batch.sync()
            rt.cudaDeviceSynchronize()
            dt = time.perf_counter() - t0
        batch.close()
        return dt, clk.summary()

    def sequential(cfgs):
        benches = [gp.DeviceBench(c, x["box"], x["first"]) for c, x in zip(cfgs, regions)]
        for t in range(W):
            for b, x in zip(benches, regions):
                b.step_device(x["steps"].value + 16 * x["n"] * t, t)
                b.sync()
        rt.cudaDeviceSynchronize()
        t0 = time.perf_counter()
        for t in range(W, total):
            for b, x in zip(benches, regions):
                b.step_device(x["steps"].value + 16 * x["n"] * t, t)
                b.sync()
        rt.cudaDeviceSynchronize()
        dt = time.perf_counter() - t0
        for b in benches:
            b.close()
        return dt

    objs = int(pops.sum())
    default_cfgs = [config(x["n"]) for x in regions]
    t_batch, clk = batched(default_cfgs)
    t_seq = sequential(default_cfgs)
    # autotune one representative region per size class
    classes = [(0, 10_000), (10_000, 100_000), (100_000, 1_000_000), (1_000_000, 1 << 40)]
    picks, tables = {}, {}
    for lo, hi in classes:
        members = [r for r in range(R) if lo <= regions[r]["n"] < hi]
        if not members:
            continue
        rep = regions[members[len(members) // 2]]

        # a trial steps through the trajectories generated above: `total`
        # steps, half of them (at most three) untimed
        tr_steps = min(6, total)
        tr_warm = tr_steps // 2

        def trial(cfg, rep=rep):
            b = gp.DeviceBench(cfg, rep["box"], rep["first"])
            for t in range(tr_warm):
                b.step_device(rep["steps"].value + 16 * rep["n"] * t, t)
                b.sync()
            rt.cudaDeviceSynchronize()
            t0 = time.perf_counter()
            for t in range(tr_warm, tr_steps):
                b.step_device(rep["steps"].value + 16 * rep["n"] * t, t)
                b.sync()
            dt = (time.perf_counter() - t0) / (tr_steps - tr_warm)
            b.close()
            return dt
        best, table = autotune(lambda cap, lf, ch, n=rep["n"]: config(n, cap, lf, ch), trial,
                               capacities=(32, 50, 128, 512, 1024), load_factors=(0.5, 0.7, 0.9),
                               chunks=(64, 128, 256, 512))
        picks[f"{lo}-{hi}"] = {"capacity": best[0], "load_factor": best[1], "refine_chunk": best[2]}
        tables[f"{lo}-{hi}"] = table
    tuned_cfgs = []
    for x in regions:
        key = next(f"{lo}-{hi}" for lo, hi in classes if lo <= x["n"] < hi)
        p = picks[key]
        tuned_cfgs.append(config(x["n"], p["capacity"], p["load_factor"], p["refine_chunk"]))
    t_tuned, _ = batched(tuned_cfgs)
    for x in regions:
        rt.cudaFree(x["steps"])
        rt.cudaFree(x["input"])
    line = {"metric": "object-timesteps/s, 64 independent regions on one GPU (batching form)",
            "value": objs * K / t_batch, "unit": UNIT, "n_gpus": 1, "steps": K, "warmup": W,
            "ms_per_step": 1000.0 * t_batch / K, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f64", "data": "synthetic",
            "config": {"workload": f"{R} regions, populations log-uniform in [1k, 2M] ({objs} objects), own street "
                                   f"grid, seed and hotspots each; reach 2 m, min meeting 5",
                       "regions": R, "objects": objs, "timing": "host wall clock around each batch step and sync"},
            "clocks": clk,
            "forms": {"batched_graphs": {"value": objs * K / t_batch, "ms_per_step": 1000.0 * t_batch / K},
                      "sequential_no_graph": {"value": objs * K / t_seq, "ms_per_step": 1000.0 * t_seq / K},
                      "batched_autotuned": {"value": objs * K / t_tuned, "ms_per_step": 1000.0 * t_tuned / K,
                                            "picks": picks}},
            "speedup_batched_vs_sequential": t_seq / t_batch,
            "parity_note": "each region's meetings equal the oracle's at the region's own leaf capacity and "
                           "buckets (the autotuned capacity changes the schema, as it would in the reference)",
            "autotune": tables}
    return line


def meeting_digest(m):
    """Order-sensitive digest of a meeting list: SHA-256 of its records
    (pid1, pid2, start, end, f32 box bits) in the order the step reported
    them."""
    import hashlib
    return hashlib.sha256(np.ascontiguousarray(m).view(np.uint8)).hexdigest()[:24]


class MeetingDigests:
    """Per-step meeting digests taken beside the stepping: each step's
    meetings are copied into one of two page-locked buffers and hashed on a
    worker thread while the next step runs (hashlib releases the GIL)."""

    def __init__(self, capacity):
        import concurrent.futures
        import glint_pipeline_gb300 as gp
        self.bufs = [gp.pinned_empty(max(1, capacity), gp.MEETING_DTYPE) for _ in range(2)]
        self.pool = concurrent.futures.ThreadPoolExecutor(max_workers=2)
        self.pending = [None, None]
        self.futs, self.counts = [], []

    def add(self, bench):
        k = len(self.futs) & 1
        if self.pending[k] is not None:
            self.pending[k].result()
        m = bench.meetings(self.bufs[k])  # a view of bufs[k], or a new array if it holds too few
        f = self.pool.submit(meeting_digest, m)
        self.pending[k] = f
        self.futs.append(f)
        self.counts.append(int(m.shape[0]))

    def result(self):
        d = [f.result() for f in self.futs]
        self.pool.shutdown()
        return d, self.counts


# the 1%-area skew: 5 hotspots whose 2-sigma discs cover 1% of the 40x40 km box
SKEW_SIGMA_SPREAD = float(np.sqrt(0.01 * 40000.0 ** 2 / (5 * np.pi)) / 2)


def run_skew(args, local, K=None, W=None):
    """Precision form on extreme skew: 20% of the objects start at 5 hotspots,
    the rest uniform over the 40x40 km street grid.  Two cases: 'spread'
    (50M objects, hotspots covering 1% of the area) for throughput, and 'core'
    (hotspots with sigma 50 m, 2M objects; at 50M objects that shape puts
    ~8e10 contacts in one step, beyond any meeting table) for the densest
    contacts.  Each case runs the plain FP64 refine and the FP32 guard-band
    refine on the same device-generated trajectories; every step's meeting
    list is compared between the two (order-sensitive digest), the band hit
    rate is the refine's in-band pairs over its distance tests, and
    glint_precision_probe gives max |d32 - d64| on sampled pairs."""
    import glint_pipeline_gb300 as gp
    from glint_pipeline_gb300 import _abi
    from glint_pipeline_gb300.tracegen import SEED_SKEW, TraceGenerator
    lib = _abi.lib()
    rt = cudart()
    rt.cudaSetDevice(local)
    K = args.steps if K is None else K
    W = max(args.warmup if W is None else W, 3)
    cases = [("spread", args.skew_objects, SKEW_SIGMA_SPREAD, args.skew_buckets, 256),
             ("core", args.core_objects, 50.0, args.core_buckets or next_pow2(256 * args.core_objects), 16)]
    out = {}
    for name, N, sigma, B, stride in cases:
        gen = TraceGenerator(SEED_SKEW, N, 1, sigma_m=sigma)
        pb, ob = gen.params_bytes(), gen.objects_bytes()  # the state before step 0
        box, first = gen.box(), gen.steps(1)[0]
        gen.close()
        res = {}
        for mode in ("plain", "tuned"):
            cfg = gp.Configuration(num_objects=N, num_meeting_buckets=B, device=local, timing=True,
                                   precision_mode=1 if mode == "tuned" else 0, auto_flush=True, store_keep=1,
                                   meeting_log_capacity=max(1 << 24, 4 * N))
            bench = gp.DeviceBench(cfg, box, first)
            gh = ctypes.c_void_p()
            assert lib.glint_gen_create(pb, len(pb), ob, N, len(ob) // N, 0, ctypes.byref(gh)) == 0
            buf = ctypes.c_void_p()
            assert rt.cudaMalloc(ctypes.byref(buf), ctypes.c_size_t(16 * N)) == 0
            digests, counts = [], []
            stage_ms = np.zeros(8)
            dev_ms, flush_ms, launches, flags = 0.0, 0.0, 0, 0
            acc = {"candidates": 0, "contacts": 0, "band_pairs": 0, "box_band": 0, "new_keys": 0, "meetings": 0}
            with Clocks(local, f"skew_{name}_{mode}") as clk:
                for t in range(W + K):
                    lib.glint_gen_step(gh, buf, ctypes.c_void_p(bench.stream))
                    bench.step_device(buf.value, t)
                    st = bench.sync()
                    flags |= st.error_flags
                    if t >= W:
                        stage_ms += np.array(st.ms)
                        dev_ms += st.ms[7] + st.flush_ms
                        flush_ms += st.flush_ms
                        launches += st.launches
                        for k in acc:
                            acc[k] += getattr(st, k)
                    m = bench.meetings()
                    digests.append(meeting_digest(m))
                    counts.append(int(m.shape[0]))
                    del m
            probe = bench.precision_probe(stride)
            lib.glint_gen_destroy(gh)
            rt.cudaFree(buf)
            bench.close()
            stage = {k: v / K for k, v in zip(STAGES, stage_ms)}
            stage["flush"] = flush_ms / K
            stage["total"] += stage["flush"]
            res[mode] = {"value": N * K / (dev_ms / 1000.0), "ms_per_step": dev_ms / K, "stage_ms": stage,
                         "per_step": {k: v / K for k, v in acc.items()}, "error_flags": flags,
                         "gpu_launches": launches, "clocks": clk.summary(), "probe": probe,
                         "_digests": digests, "meetings_per_step": counts}
        dp, dt = res["plain"].pop("_digests"), res["tuned"].pop("_digests")
        steps_differ = [t for t in range(len(dp)) if dp[t] != dt[t] or
                        res["plain"]["meetings_per_step"][t] != res["tuned"]["meetings_per_step"][t]]
        tu = res["tuned"]["per_step"]
        out[name] = {"objects": N, "sigma_m": sigma, "buckets": B, "forms": res,
                     "meetings_compared": int(sum(res["plain"]["meetings_per_step"])),
                     "steps_compared": len(dp), "steps_differing": steps_differ,
                     "band_hit_rate": tu["band_pairs"] / max(tu["candidates"], 1),
                     "box_band_per_step": tu["box_band"],
                     "speedup_tuned_vs_plain": res["plain"]["ms_per_step"] / res["tuned"]["ms_per_step"]}
    sp = out["spread"]
    head = sp["forms"]["tuned"]
    line = {"metric": "object-timesteps/s, precision form (FP32 guard band) on extreme skew, meetings equal to "
                      "the FP64 form",
            "value": head["value"], "unit": UNIT, "n_gpus": 1, "steps": K, "warmup": W,
            "ms_per_step": head["ms_per_step"], "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f64+f32", "data": "synthetic",
            "config": {"workload": f"Manhattan-grid generator, 40x40 km: {sp['objects']} objects, 20% at 5 "
                                   f"hotspots (sigma {SKEW_SIGMA_SPREAD:.0f} m: 1% of the area), reach 2 m, "
                                   f"min meeting 5, {sp['buckets']} buckets; plus a sigma 50 m core case of "
                                   f"{out['core']['objects']} objects",
                       "l2": "inputs larger than L2"},
            "clocks": head["clocks"], "gpu_launches": head["gpu_launches"], "cases": out}
    return line


def main():
    args = parse()
    rank, world, local, pg = dist_init()
    if args.impl == "reference":
        run_reference_arm(args, rank, world, pg)
        return
    if args.workload == "batch64":
        if rank == 0:
            print(json.dumps(run_batch(args, local)), flush=True)
        return
    if args.workload == "skew50m":
        if rank == 0:
            print(json.dumps(run_skew(args, local)), flush=True)
        return
    if args.workload == "serve":
        if rank == 0:
            from glint_pipeline_gb300.tracegen import SEED_SCALE, TraceGenerator
            g = TraceGenerator(SEED_SCALE, args.objects)
            box, first = g.box(), g.steps(1)[0]
            g.close()
            g2 = TraceGenerator(SEED_SCALE, args.objects)
            pb, ob = g2.params_bytes(), g2.objects_bytes()
            g2.close()
            res = serving_store(args, local, args.objects, pb, ob, box, first)
            print(json.dumps({"workload": "serve", "metric": "query latency over a store of --serve-steps steps",
                              "serving": res}), flush=True)
        return
    if args.workload == "compact":
        if rank == 0:
            res = compaction_sample(args, local)
            print(json.dumps({"workload": "compact", "metric": "source keys/s merged into split_num^2 CTFs",
                              "compaction": res}), flush=True)
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
    serve = compact = None
    for m in modes:
        forms[m] = run_form(args, m, N, local, pg, world, box, first, pb, ob, dbuf, step_bytes, rt)
        b = forms[m].pop("_bench")
        if m == modes[0] and not args.no_compact:
            compact = compaction(args, b)
            if compact and "error" not in compact and not args.no_serve:
                # the same query stream over the one merged block: a query
                # scans the same keys, now in one block instead of several
                compact["serving"] = serving(args, b, N, total, sweep_rates=False)
        b.close()
    rt.cudaFree(dbuf)
    if not args.no_serve and world == 1:
        try:
            serve = serving_store(args, local, N, pb, ob, box, first)
        except Exception as e:  # reported in the line; the headline does not depend on it
            serve = {"error": f"{type(e).__name__}: {e}"}
    other = {}
    if not args.no_forms and world == 1:
        # the batching and precision forms, a few steps each (their own
        # --workload runs give the full lines)
        for name, fn in (("batch64", run_batch), ("skew50m", run_skew)):
            t0 = time.perf_counter()
            try:
                other[name] = fn(args, local, K=args.form_steps, W=3)
            except Exception as e:  # reported in the line; the headline does not depend on it
                other[name] = {"error": f"{type(e).__name__}: {e}"}
            other[name]["wall_s"] = time.perf_counter() - t0
    head = forms[modes[0]]
    parity = {}
    if len(modes) == 2:
        dt_, dp_ = forms["tuned"]["_digests"], forms["plain"]["_digests"]
        ct_, cp_ = forms["tuned"]["_meetings"], forms["plain"]["_meetings"]
        parity["tuned_vs_plain"] = {
            "steps": len(dt_), "meetings": int(sum(ct_)), "timed_steps": K,
            "mismatching_steps": [t for t in range(min(len(dt_), len(dp_))) if dt_[t] != dp_[t] or ct_[t] != cp_[t]],
            "compared": "every step (warm-up and timed) of the two forms on the same trajectories: meetings "
                        "(pid1, pid2, start, end, f32 box bits) in bucket order, SHA-256"}
    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu:
        cpu = cpu_baseline(args, N, args.buckets, args.cpu_steps, args.cpu_warmup, head["_digests"])
        if "parity" in cpu:
            parity["oracle"] = cpu.pop("parity")
    if compact is not None and rank == 0 and world == 1 and not args.no_cpu:
        compact["sample"] = compaction_sample(args, local)
    for f in forms.values():
        f.pop("_digests", None)
        f.pop("_meetings", None)
    if rank == 0:
        line = {"metric": METRIC, "value": head["value"], "unit": UNIT, "n_gpus": world, "steps": K, "warmup": W,
                "ms_per_step": head["ms_per_step"], "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
                "dtype": "f64", "data": "synthetic", "config": workload_config(args, N, modes[0]),
                "roofline": roofline(head, N, args.buckets, modes[0]), "clocks": head["clocks"], "e2e": head["e2e"],
                "cpu_baseline": cpu, "parity": parity,
                "gpu_launches": head["gpu_launches"], "serving": serve, "compaction": compact,
                "forms": dict({m: {k: v for k, v in f.items()} for m, f in forms.items()}, **other)}
        bad = {k: v["mismatching_steps"] for k, v in parity.items() if v.get("mismatching_steps")}
        line["parity_ok"] = not bad
        print(json.dumps(line), flush=True)
        if bad:
            # the line above carries the numbers; a run whose meetings differ fails
            print(f"meetings differ on steps {bad}", file=sys.stderr)
            sys.exit(3)


if __name__ == "__main__":
    main()
