"""The C++ shim defines the reference's GPU seam with the reference's own
signatures: compiled against the reference headers it exports exactly the
symbols that the reference's process.cpp (built with USE_GPU) leaves
undefined, and it links against libglint.so.  CPU only; skipped where the
reference sources are absent."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REF = os.environ.get("GLINT_REFERENCE_ROOT", "/root/reference")
SRC = os.path.join(REF, "src")
SHIM = os.path.join(ROOT, "glint_pipeline_gb300", "shim", "glint_ref_shim.cpp")
CUDA_INC = os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "include")

pytestmark = pytest.mark.skipif(not os.path.isdir(os.path.join(SRC, "tracing")) or shutil.which("g++") is None,
                                reason="reference sources or g++ not available")

SEAM = ("_Z24cuda_create_device_benchP9workbenchP8gpu_info", "_Z16process_with_gpuP9workbenchS0_P8gpu_info")


def _flags():
    # the Boost stub stands in for program_options, which util/config.h includes
    return ["-std=c++17", "-O1", "-fPIC", "-w", "-I" + os.path.join(ROOT, "oracle", "ref_stub"), "-I" + SRC,
            "-I" + CUDA_INC, "-I" + os.path.join(ROOT, "include")]


def _symbols(obj):
    out = subprocess.run(["nm", obj], capture_output=True, text=True, check=True).stdout
    syms = {}
    for line in out.splitlines():
        parts = line.split()
        if len(parts) >= 2:
            syms[parts[-1]] = parts[-2]
    return syms


def test_shim_matches_reference_seam(tmp_path):
    shim_o = str(tmp_path / "shim.o")
    proc_o = str(tmp_path / "process.o")
    subprocess.run(["g++", *_flags(), "-c", SHIM, "-o", shim_o], check=True)
    subprocess.run(["g++", *_flags(), "-DUSE_GPU", "-c", os.path.join(SRC, "tracing", "process.cpp"), "-o", proc_o],
                   check=True)
    shim, proc = _symbols(shim_o), _symbols(proc_o)
    for s in SEAM:
        assert proc.get(s) == "U", f"process.cpp does not call {s}"
        assert shim.get(s) == "T", f"shim does not define {s}"


def test_shim_links_against_libglint(tmp_path):
    from glint_pipeline_gb300 import build
    lib = build.build()
    shim_o = str(tmp_path / "shim.o")
    subprocess.run(["g++", *_flags(), "-c", SHIM, "-o", shim_o], check=True)
    so = str(tmp_path / "libshim.so")
    subprocess.run(["g++", "-shared", "-o", so, shim_o, "-L" + os.path.dirname(lib), "-lglint",
                    "-Wl,--no-undefined", "-Wl,--unresolved-symbols=ignore-in-object-files"], check=True)
    undefined = [s for s, k in _symbols(shim_o).items() if k == "U" and s.startswith("glint_")]
    exported = subprocess.run(["nm", "-D", "--defined-only", lib], capture_output=True, text=True).stdout
    for s in undefined:
        assert s in exported, s
