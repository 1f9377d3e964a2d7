"""In-tree build of the native libraries.

libglint.so      every CUDA kernel and the C ABI (include/glint.h), sm_103a only
_tracegen.so     the host side of the synthetic trajectory generator

Compiled with nvcc / gcc directly (no cmake): one nvcc process per
translation unit, run in parallel, then one link.  Host code is compiled with
-ffp-contract=off so FP64 expressions are rounded once per operation on both
x86-64 and aarch64 hosts.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
INCLUDE = os.path.join(ROOT, "include")
BUILD_DIR = os.path.join(HERE, "_build")
LIBGLINT = os.path.join(HERE, "libglint.so")
TRACEGEN = os.path.join(HERE, "_tracegen.so")

CU_SOURCES = ["glint_api.cu", "k_util.cu", "k_partition.cu", "k_filter.cu", "k_refine.cu", "k_identify.cu",
              "k_schema.cu", "k_precision.cu", "k_flush.cu", "k_query.cu", "k_sort.cu",
              "k_serve.cu", "glint_batch.cu", "store_files.cu",
              "glint_pipe.cu", "trace_files.cu", "snapshot.cu", "k_compact.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc_path() -> str:
    cuda = os.environ.get("CUDA_HOME", "/usr/local/cuda")
    p = os.path.join(cuda, "bin", "nvcc")
    return p if os.path.exists(p) else (shutil.which("nvcc") or "nvcc")


def _headers():
    out = []
    for d in (CSRC, INCLUDE):
        for f in os.listdir(d):
            if f.endswith((".h", ".cuh")):
                out.append(os.path.join(d, f))
    return out


def _stale(target: str, deps) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps if os.path.exists(d))


def _compile(src: str, verbose: bool) -> str:
    obj = os.path.join(BUILD_DIR, os.path.basename(src) + ".o")
    if not _stale(obj, [src, __file__] + _headers()):
        return obj
    cmd = [nvcc_path(), *ARCH, "-O3", "-lineinfo", "-std=c++17", "-c", src, "-o", obj,
           "-I", CSRC, "-I", INCLUDE, "-Xcompiler", "-fPIC,-ffp-contract=off", "--expt-relaxed-constexpr"]
    if verbose:
        print(" ".join(cmd), flush=True)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{r.stdout}\n{r.stderr}")
    return obj


def build_tracegen(verbose: bool = False) -> str:
    src = os.path.join(CSRC, "tracegen_host.c")
    if _stale(TRACEGEN, [src, os.path.join(CSRC, "tracegen.h")]):
        cc = os.environ.get("CC", "gcc")
        cmd = [cc, "-O2", "-ffp-contract=off", "-fPIC", "-shared", "-o", TRACEGEN, src, "-lm"]
        if verbose:
            print(" ".join(cmd), flush=True)
        subprocess.run(cmd, check=True)
    return TRACEGEN


def build_glint(verbose: bool = False) -> str:
    os.makedirs(BUILD_DIR, exist_ok=True)
    srcs = [os.path.join(CSRC, s) for s in CU_SOURCES]
    with cf.ThreadPoolExecutor(max_workers=min(len(srcs), os.cpu_count() or 4)) as ex:
        objs = list(ex.map(lambda s: _compile(s, verbose), srcs))
    if _stale(LIBGLINT, objs):
        cmd = [nvcc_path(), *ARCH, "-shared", "-o", LIBGLINT, *objs, "-Xcompiler", "-fPIC"]
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    return LIBGLINT


def build(verbose: bool = False):
    build_tracegen(verbose)
    return build_glint(verbose)


if __name__ == "__main__":
    build(verbose="-v" in sys.argv)
    print(LIBGLINT)
