"""Check and time the reference's own GPU kernel (rng_outer_32 of
cuda/mrg8_cuda.cu:282-399) on this GPU.  TEST INFRASTRUCTURE ONLY.

Needs oracle/_ref/mrg8_ref_cuda.cubin, which `make -C oracle refcubin`
compiles from the reference sources (where they are present); builds its own
loader (`make -C oracle refgpu`).  Prints one JSON line:

    python oracle/ref_gpu_run.py [--n-check 2^24] [--n 2^30] [--reps 10]

`check`: the kernel's outputs (rng_outer_32, and rng_inner of
cuda/mrg8_cuda.cu:201-280) for seed 13579 at the reference's default launch
shape (65,536 threads in blocks of 64) against the oracle's SHIFTED fp64
stream, bit for bit, and its next state.  `time`: the kernel alone (CUDA
events around the launches, no allocation or copy of the reference's host
wrapper) over the launch shapes the reference's own driver sweeps
(cuda/tests/test_mrg8_outer.cu:51-78), at n outputs.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
CUBIN = os.path.join(HERE, "_ref", "mrg8_ref_cuda.cubin")
DRIVER = os.path.join(HERE, "_build", "ref_gpu_driver")
SEED = 13579


def available() -> bool:
    return os.path.exists(CUBIN)


def build_driver() -> None:
    subprocess.run(["make", "-s", "-C", HERE, "refgpu"], check=True)


def check(n: int, tnum: int = 64 * 1024, bs: int = 64, kernel: str = "outer") -> dict:
    sys.path.insert(0, os.path.dirname(HERE))
    from oracle.pyoracle import F64_SHIFTED, Oracle
    o = Oracle()
    with tempfile.TemporaryDirectory() as d:
        path = os.path.join(d, "out.bin")
        subprocess.run([DRIVER, CUBIN, "check", str(n), str(SEED), str(tnum), str(bs), path, kernel], check=True)
        raw = np.fromfile(path, dtype=np.uint8)
    got = raw[: 8 * n].view(np.float64)
    nxt = raw[8 * n:].view(np.uint32)
    st = o.seed(SEED)
    want, end = o.generate(st, n, F64_SHIFTED, nthreads=os.cpu_count() or 4)
    diff = int(np.count_nonzero(got.view(np.uint64) != want.view(np.uint64)))
    return {"kernel": kernel, "n": n, "tnum": tnum, "bs": bs, "mismatches": diff,
            "next_state_equal": bool(np.array_equal(nxt, end))}


def time_shapes(n: int, reps: int, shapes, kernel: str = "outer") -> list:
    rows = []
    for tnum, bs in shapes:
        r = subprocess.run([DRIVER, CUBIN, "time", str(n), str(SEED), str(tnum), str(bs), str(reps), kernel],
                           capture_output=True, text=True, check=True)
        t, b, nn, ms, gs = r.stdout.split()
        rows.append({"tnum": int(t), "bs": int(b), "ms": float(ms), "gsamples_per_s": float(gs)})
    return rows


def main() -> int:
    ap = argparse.ArgumentParser()
    ap.add_argument("--n-check", type=int, default=1 << 24)
    ap.add_argument("--n", type=int, default=1 << 30)
    ap.add_argument("--reps", type=int, default=10)
    args = ap.parse_args()
    if not available():
        print(json.dumps({"reference_gpu": "unavailable", "why": f"{CUBIN} not built (no reference sources)"}))
        return 0
    build_driver()
    chk = check(args.n_check)
    shapes = [(t, b) for t in (64 * 1024, 256 * 1024, 1024 * 1024) for b in (32, 64, 128, 256, 512)]
    rows = time_shapes(args.n, args.reps, shapes)
    best = max(rows, key=lambda r: r["gsamples_per_s"])
    default = next(r for r in rows if r["tnum"] == 64 * 1024 and r["bs"] == 64)
    chk_in = check(args.n_check, kernel="inner")
    rows_in = time_shapes(args.n, max(1, args.reps // 5), [(t, 64) for t in (64 * 1024, 1024 * 1024)], "inner")
    print(json.dumps({"reference_gpu": "rng_outer_32", "check": chk, "n": args.n, "default_shape": default,
                      "best_shape": best, "all": rows,
                      "rng_inner": {"check": chk_in, "shapes": rows_in}}))
    return 0


if __name__ == "__main__":
    sys.exit(main())
