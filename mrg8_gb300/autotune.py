"""Launch-shape autotuner for the bulk kernel.

For each output kind it times the bulk kernel over the candidate layouts
(V = 1, 2 or 4 substreams per lane, i.e. outputs per thread per row) and
resident blocks per SM (occupancy caps), with CUDA events on the launch
stream, and applies the fastest through ``mrg8g_tune_plain``.  Results can be
cached in a JSON file keyed by the GPU name (``MRG8G_TUNE_CACHE`` or the
``cache`` argument).  Tuning never changes the generated values: every shape
produces the same stream.
"""
from __future__ import annotations

import ctypes as C
import json
import os

from . import _lib
from ._lib import F32_ORIGINAL, F32_SHIFTED, F64_ORIGINAL, F64_SHIFTED, U32, check

KIND_NAMES = {U32: "u32", F64_ORIGINAL: "f64_original", F64_SHIFTED: "f64_shifted",
              F32_ORIGINAL: "f32_original", F32_SHIFTED: "f32_shifted"}


def _device_name(torch) -> str:
    return torch.cuda.get_device_name(torch.cuda.current_device())


def time_plain(kind: int, n: int, V: int, bps: int, reps: int = 5, out=None) -> float:
    """Seconds per bulk launch of n outputs with the given shape."""
    import torch

    from .api import MRG8
    lib = _lib.load()
    check(lib.mrg8g_tune_plain(kind, V, bps))
    dt = torch.float64 if kind in (F64_ORIGINAL, F64_SHIFTED) else (torch.int32 if kind == U32 else torch.float32)
    if out is None:
        out = torch.empty(n, dtype=dt, device="cuda")
    g = MRG8(13579)
    st = g.get_state()
    stream = torch.cuda.current_stream()
    for _ in range(2):
        g.set_state(st)
        g._generate(out, n, kind)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(reps):
        g.set_state(st)
        g._generate(out, n, kind)
    e1.record(stream)
    torch.cuda.synchronize()
    return e0.elapsed_time(e1) / 1e3 / reps


def tune_plain(kinds=(F64_SHIFTED, F64_ORIGINAL, F32_SHIFTED, F32_ORIGINAL, U32), n: int = 1 << 28,
               layouts=(1, 2, 4), occupancies=(0, 4, 6, 8, 12), cache: str | None = None,
               verbose: bool = False) -> dict:
    """Pick and apply the fastest (V, blocks per SM) per kind; returns
    {kind name: {"V":, "blocks_per_sm":, "gsamples_per_s":}}."""
    import torch
    lib = _lib.load()
    cache = cache or os.environ.get("MRG8G_TUNE_CACHE")
    name = _device_name(torch)
    if cache and os.path.exists(cache):
        with open(cache) as f:
            saved = json.load(f).get(name)
        if saved and all(KIND_NAMES[k] in saved for k in kinds):
            for k in kinds:
                r = saved[KIND_NAMES[k]]
                check(lib.mrg8g_tune_plain(k, r["V"], r["blocks_per_sm"]))
            return saved
    result = {}
    bufs = {}
    for k in kinds:
        dt = torch.float64 if k in (F64_ORIGINAL, F64_SHIFTED) else (torch.int32 if k == U32 else torch.float32)
        if dt not in bufs:
            bufs[dt] = torch.empty(n, dtype=dt, device="cuda")
        best = None
        for V in layouts:
            for bps in occupancies:
                t = time_plain(k, n, V, bps, out=bufs[dt])
                if verbose:
                    print(f"  {KIND_NAMES[k]:13s} V={V} bps={bps:2d}: {n / t / 1e9:8.1f} Gsamples/s")
                if best is None or t < best[0]:
                    best = (t, V, bps)
        check(lib.mrg8g_tune_plain(k, best[1], best[2]))
        result[KIND_NAMES[k]] = {"V": best[1], "blocks_per_sm": best[2], "gsamples_per_s": n / best[0] / 1e9}
    if cache:
        data = {}
        if os.path.exists(cache):
            with open(cache) as f:
                data = json.load(f)
        data[name] = result
        with open(cache, "w") as f:
            json.dump(data, f, indent=1)
    return result


def current_plain_tuning() -> dict:
    lib = _lib.load()
    out = {}
    for k, nm in KIND_NAMES.items():
        V, b = C.c_int(), C.c_int()
        check(lib.mrg8g_get_plain_tuning(k, C.byref(V), C.byref(b)))
        out[nm] = {"V": V.value, "blocks_per_sm": b.value}
    return out


if __name__ == "__main__":
    print(json.dumps(tune_plain(verbose=True), indent=1))
