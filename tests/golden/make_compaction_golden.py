"""Generates tests/golden/compaction.npz from the reference's own compaction.

Writes flushed blocks of seeded oracle runs in the reference's file layout
under tests/.tmp, runs the unmodified merge_dump (tools/compaction.cpp, built
by oracle/build_ref.sh into oracle/_ref) over them, and records what the
reference wrote: sids, CTF records, and digests of the packed keys, the
bitmaps and the oversize buffer.  Only this script runs the reference; the
committed fixture travels to machines without it.

    python tests/golden/make_compaction_golden.py
"""
from __future__ import annotations

import os
import shutil
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
TESTS = os.path.dirname(HERE)
ROOT = os.path.dirname(TESTS)
sys.path.insert(0, ROOT)
sys.path.insert(0, TESTS)

from glint_pipeline_gb300 import write_store_files  # noqa: E402
from oracle.bindings import build_ref  # noqa: E402
from test_compact_oracle import CASES, read_reference, run_reference, source_blocks  # noqa: E402
from workloads import digest  # noqa: E402

# (case, split_num) pairs recorded in the fixture
GOLDEN = [("object0", 3), ("oversize", 4), ("dense", 5)]


def reference_result(case, split_num, work):
    box, blocks = source_blocks(**CASES[case])
    n = blocks[0][1]["sids"].shape[0]
    if os.path.isdir(work):
        shutil.rmtree(work)
    for d in ("r0", "r1", "m"):
        os.makedirs(os.path.join(work, d))
    for i, (info, b) in enumerate(blocks):
        write_store_files(b, info, n, os.path.join(work, "r"), os.path.join(work, "m"), "src", i)
    run_reference(work, len(blocks), n, 100, box, split_num)
    C = split_num * split_num
    cwd = os.getcwd()
    os.chdir(work)
    try:
        # sizes for the readers' buffers: a generous bound on the key bytes
        bound = {"o_count": sum(int(b["o_keys"].shape[0]) for _, b in blocks),
                 "key_bytes": sum(int(b["keys"].size) for _, b in blocks) * 2,
                 "ctfs": blocks[0][1]["ctfs"]}
        ref = read_reference(len(blocks), n, C, bound)
    finally:
        os.chdir(cwd)
    return ref, C


def record(ref, C):
    ctfs = ref["ctfs"]
    cap = ctfs["CTF_kv_capacity"].astype(np.int64)
    key_bytes = int((cap * (ctfs["key_bit"].astype(np.int64) // 8)).sum())
    on = int(ref["ot"][0])
    bits = np.concatenate([ref["bitmaps"][c * 8192:c * 8192 + int(ctfs["ctf_bitmap_size"][c])] for c in range(C)])
    return dict(sids=ref["sids"], ctfs=ctfs.view(np.uint8).ravel().copy(), ot=ref["ot"],
                keys_digest=np.array(digest(ref["keys"][:key_bytes])), bitmaps_digest=np.array(digest(bits)),
                o_digest=np.array(digest(ref["o_keys"][:on], ref["o_boxes"][:on].view(np.uint32), ref["o_bitmap"])))


def main():
    if build_ref() is None:
        raise SystemExit("the reference sources are not present on this machine")
    out = {}
    work = os.path.join(TESTS, ".tmp", "compaction_golden")
    for case, s in GOLDEN:
        ref, C = reference_result(case, s, work)
        for k, v in record(ref, C).items():
            out[f"{case}_{s}_{k}"] = v
        print(f"{case} split_num {s}: {int(ref['ctfs']['CTF_kv_capacity'].sum())} keys")
    shutil.rmtree(work, ignore_errors=True)
    np.savez_compressed(os.path.join(HERE, "compaction.npz"), **out)


if __name__ == "__main__":
    main()
