"""Times the reference's own CPU stages against the oracle's C restatement on
one host, on the same seeded workload, so that the restatement's figure on a
machine without the reference (where bench.py times it as the CPU baseline)
can be read as the reference's.

TEST INFRASTRUCTURE: runs where the reference's sources are (it builds them
with oracle/build_ref.sh).  Each variant runs in a child process of its own:

  reference -O2         oracle/_ref/libglintref.so (build_ref.sh defaults)
  reference as shipped  oracle/_ref/libglintref_asshipped.so (src/Makefile:13
                        flags: -g, no -O), built here when missing
  port                  oracle/liboracle.so (the oracle, -O2)

with 1 thread and with every host thread.  The per-step sequence of the
reference's variants is tracer::process's CPU branch (tracing/process.cpp:
453-459: filter, reachability, update_meetings, update_schema), whose filter
and reachability loops run on config->num_threads OpenMP threads
(tracing/workbench.cpp:356,581).

  usage: python oracle/calibrate_cpu.py [--objects N] [--buckets B]
             [--steps K] [--out FILE]
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import time

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
ASSHIPPED = os.path.join(HERE, "_ref", "libglintref_asshipped.so")


def one(kind: str, threads: int, N: int, B: int, steps: int, warm: int) -> dict:
    sys.path.insert(0, ROOT)
    from glint_pipeline_gb300.tracegen import SEED_SCALE, TraceGenerator
    from oracle.bindings import Oracle, Reference, make_config
    g = TraceGenerator(SEED_SCALE, N)
    box, pts = g.box(), g.steps(warm + steps)
    g.close()
    cfg = make_config(N, num_meeting_buckets=B)
    t0 = time.perf_counter()
    if kind == "port":
        o = Oracle(cfg, box, pts[0], threads=threads)
    else:
        o = Reference(cfg, box, pts[0], num_threads=threads)
    create_s = time.perf_counter() - t0
    times, meetings = [], 0
    for t in range(warm + steps):
        t0 = time.perf_counter()
        o.step(pts[t], t)
        dt = time.perf_counter() - t0
        if t >= warm:
            times.append(dt)
            meetings += int(o.counts().kv_count)
    o.close()
    return {"kind": kind, "threads": threads, "objects": N, "buckets": B, "steps": steps, "warmup": warm,
            "create_s": create_s, "ms_per_step": 1000.0 * sum(times) / len(times),
            "step_ms": [1000.0 * x for x in times], "meetings": meetings}


def cpu_model() -> str:
    for line in open("/proc/cpuinfo"):
        if line.startswith("model name"):
            return line.split(":", 1)[1].strip()
    return "unknown"


def main():
    p = argparse.ArgumentParser()
    p.add_argument("--objects", type=int, default=10_000_000)
    p.add_argument("--buckets", type=int, default=1 << 30)
    p.add_argument("--steps", type=int, default=2)
    p.add_argument("--warmup", type=int, default=1)
    p.add_argument("--out", default=os.path.join(ROOT, "profiles", "cpu_reference_vs_port.md"))
    p.add_argument("--one", default=None, help=argparse.SUPPRESS)
    p.add_argument("--threads", type=int, default=1, help=argparse.SUPPRESS)
    a = p.parse_args()
    if a.one:
        print(json.dumps(one(a.one, a.threads, a.objects, a.buckets, a.steps, a.warmup)), flush=True)
        return
    sys.path.insert(0, ROOT)
    from oracle.bindings import REFERENCE_ROOT, build_oracle, build_ref
    build_oracle()
    if build_ref() is None:
        sys.exit("the reference's sources are not on this machine")
    if not os.path.exists(ASSHIPPED):
        env = dict(os.environ, REF_OPT="-g", REF_LIB=os.path.basename(ASSHIPPED), REF_CPU_ONLY="1")
        subprocess.run(["sh", os.path.join(HERE, "build_ref.sh"), REFERENCE_ROOT], check=True, env=env,
                       stdout=subprocess.DEVNULL)
    nthreads = os.cpu_count() or 1
    variants = [("reference -O2", "ref", None), ("reference as shipped (-g)", "ref", ASSHIPPED),
                ("port (oracle, -O2)", "port", None)]
    rows = []
    for label, kind, lib in variants:
        for threads in sorted({1, nthreads}):
            env = dict(os.environ)
            if lib:
                env["GLINT_REF_SO"] = lib
            cmd = [sys.executable, os.path.abspath(__file__), "--one", kind, "--threads", str(threads),
                   "--objects", str(a.objects), "--buckets", str(a.buckets), "--steps", str(a.steps),
                   "--warmup", str(a.warmup)]
            r = subprocess.run(cmd, env=env, capture_output=True, text=True)
            if r.returncode != 0:
                rows.append({"label": label, "threads": threads, "error": r.stderr.strip().splitlines()[-1:]})
                continue
            res = json.loads(r.stdout.strip().splitlines()[-1])
            res["label"] = label
            rows.append(res)
            print(json.dumps(res), flush=True)
    base = {r["threads"]: r["ms_per_step"] for r in rows if r.get("label") == "reference -O2" and "ms_per_step" in r}
    lines = ["# CPU stages: the reference's own code against the oracle's restatement, one host", "",
             "Command (where the reference's sources are; each variant in its own process):", "", "```",
             f"python oracle/calibrate_cpu.py --objects {a.objects} --buckets {a.buckets} --steps {a.steps} "
             f"--warmup {a.warmup}", "```", "",
             f"Host: {cpu_model()}, {nthreads} threads.  Workload: the seeded Manhattan-grid generator at "
             f"{a.objects} objects, {a.buckets} buckets, leaf capacity 50, reach 2 m, min meeting 5; "
             f"steps {a.warmup}..{a.warmup + a.steps - 1} timed after {a.warmup} untimed.", "",
             "| variant | threads | ms per step | vs reference -O2, same threads | meetings |",
             "|---|---:|---:|---:|---:|"]
    for r in rows:
        if "ms_per_step" not in r:
            lines.append(f"| {r['label']} | {r['threads']} | failed: {r['error']} | | |")
            continue
        ref_ms = base.get(r["threads"])
        ratio = f"{ref_ms / r['ms_per_step']:.2f}x" if ref_ms else ""
        lines.append(f"| {r['label']} | {r['threads']} | {r['ms_per_step']:.0f} | {ratio} | {r['meetings']} |")
    lines += ["", "The ratio column is the reference -O2's time over the variant's: above 1 the variant is faster.",
              "The reference with more than one thread orders its table inserts by thread timing; its meeting "
              "counts can then differ from one thread's, the port's do not."]
    with open(a.out, "w") as f:
        f.write("\n".join(lines) + "\n")
    print(f"wrote {a.out}")


if __name__ == "__main__":
    main()
