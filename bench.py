"""Benchmark of the MRG8 bulk path on GB300 (one JSON line on rank 0).

Workload (one step): the plain single-stream generator writes 2^30 fp64
uniforms (SHIFTED scaling, [0,1), as cuda/mrg8_cuda.cu's mrg8_outer_32) from
seed 13579 into an HBM-resident buffer: one launch of the bulk kernel.  The
output (8 GiB) is larger than L2, so no flush is needed between steps.

  value    whole-job Gsamples/s, device buffer, CUDA events on the launch stream
  e2e      the same through the C ABI with a pinned HOST buffer
           (mrg8g_generate_host: device staging + D2H inside the timed region)
  roofline HBM-write roofline of the bulk kernel against MEASURED_PEAKS.json
  f32      fp32 SHIFTED at the same size, and (other_kinds) uint32, fp64
           ORIGINAL and fp32 ORIGINAL
  cpu_baseline  the reference's CPU paths on the host: the block-split
           generator on all cores (knl/mrg8_vec.h:500-525) and the scalar
           sequential rand() of original/mrg8.cpp:231-239 on one core,
           both through the oracle's restatement
  batched  config 4: one batch launch vs one bulk launch per instance
  jump_stress  config 3: 65,536 device jumps by offsets in [0, 2^63), and
           4,096 uint32 outputs after each in one batch launch
  served   config 5: Poisson 20k req/s for 60 s, plus a short rate sweep

``--impl reference`` times the reference's CPU implementation of the path
(the build in oracle/_ref where it exists, else the oracle port) on the same
metric and workload (2^30 outputs per step), and, where the reference's GPU
kernel was compiled from its sources (oracle/_ref/mrg8_ref_cuda.cubin), checks
that kernel against the oracle and times it on this GPU with a clock record
(``ref_gpu``; not part of ``value``).  Under torchrun each rank generates its
own 2^30-output shard of one stream (rank r starts r * 2^30 outputs in; no
collective on the data path).
"""
from __future__ import annotations

import argparse
import json
import os
import re
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

SEED = 13579
N_PER_RANK = 1 << 30
METRIC = "fp64 Gsamples/s & %HBM peak at 2^30; batched vs per-call speedup; served p50/p99"
UNIT = "Gsamples/s"
WORKLOAD = "plain MRG8 single stream: 2^30 fp64 uniforms (SHIFTED, [0,1)) from seed 13579 per GPU"
CPU_SAMPLE_N = 1 << 28
SCALAR_SAMPLE_N = 1 << 26


def workload_config(n: int, ws: int) -> dict:
    """The `config` of both arms' lines (same keys and values)."""
    return {"workload": WORKLOAD, "n": n, "seed": SEED,
            "l2": "each step writes 8 GiB (> 129 MB L2): no flush needed", "parallelism": f"shard{ws}"}


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def measured_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return json.load(f), "measured"
    except OSError:
        return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0}, "fallback"


def profiled_traffic(name: str):
    """Per-launch DRAM bytes recorded from an ncu capture in profiles/<name>."""
    path = os.path.join(ROOT, "profiles", name)
    try:
        text = open(path).read()
    except OSError:
        return None
    m = re.search(r"traffic_bytes_per_launch:\s*([0-9.eE+]+)", text)
    return float(m.group(1)) if m else None


def gpu_id(index: int) -> str:
    """nvidia-smi / NVML identity of CUDA device `index` (its UUID), so that a
    restricted CUDA_VISIBLE_DEVICES still samples the GPU under test."""
    try:
        import torch
        u = str(torch.cuda.get_device_properties(index).uuid)
        return u if u.startswith("GPU-") else "GPU-" + u
    except Exception:
        return str(index)


class NvmlClockSampler:
    """SM clock and clock-event reasons read through NVML (read-only queries)
    every millisecond on a background thread, so that even a timed region of a
    few tens of milliseconds holds many samples.  Falls back to nothing when
    the NVML library cannot be loaded."""

    REASONS = {0x4: "sw_power_cap", 0x8: "hw_slowdown", 0x20: "sw_thermal_slowdown", 0x40: "hw_thermal_slowdown",
               0x80: "hw_power_brake_slowdown"}

    def __init__(self, index: int, period_s: float = 1e-3):
        import ctypes as C
        self.C = C
        self.period = period_s
        self.samples = []
        self.ok = False
        try:
            lib = C.CDLL("libnvidia-ml.so.1")
            if lib.nvmlInit_v2() != 0:
                return
            h = C.c_void_p()
            ident = gpu_id(index)
            rc = (lib.nvmlDeviceGetHandleByUUID(ident.encode(), C.byref(h)) if ident.startswith("GPU-")
                  else lib.nvmlDeviceGetHandleByIndex_v2(C.c_uint(int(ident)), C.byref(h)))
            if rc != 0:
                return
            mx = C.c_uint()
            self.max_mhz = float(mx.value) if lib.nvmlDeviceGetMaxClockInfo(h, 1, C.byref(mx)) == 0 else None
            self.reasons_fn = getattr(lib, "nvmlDeviceGetCurrentClocksEventReasons", None) or \
                lib.nvmlDeviceGetCurrentClocksThrottleReasons
            self.lib, self.h, self.ident = lib, h, ident
            self.ok = True
        except (OSError, AttributeError):
            self.ok = False

    def _run(self):
        C = self.C
        clk, rs = C.c_uint(), C.c_ulonglong()
        while not self.stop:
            a = self.lib.nvmlDeviceGetClockInfo(self.h, 1, C.byref(clk))
            b = self.reasons_fn(self.h, C.byref(rs))
            if a == 0:
                self.samples.append((float(clk.value), int(rs.value) if b == 0 else 0))
            time.sleep(self.period)

    def __enter__(self):
        import threading
        self.stop = False
        if self.ok:
            self.thread = threading.Thread(target=self._run, daemon=True)
            self.thread.start()
        return self

    def __exit__(self, *exc):
        self.stop = True
        if self.ok:
            self.thread.join()

    def summary(self):
        if not self.ok or not self.samples:
            return None
        sm = [c for c, _ in self.samples]
        reasons = sorted({name for _, r in self.samples for bit, name in self.REASONS.items() if r & bit})
        loaded = [v for v in sm if self.max_mhz and v > 0.5 * self.max_mhz] or sm
        return {"sm_mhz": statistics.median(loaded), "sm_max_mhz": self.max_mhz, "reasons": reasons,
                "samples": len(sm), "source": "nvml, 1 ms", "gpu": self.ident}


class ClockSampler:
    """Clocks and throttle reasons during the timed region: NVML every
    millisecond where it loads, else nvidia-smi every 200 ms."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.tmp = None
        self.nvml = NvmlClockSampler(index)

    def __enter__(self):
        if self.nvml.ok:
            self.nvml.__enter__()
            return self
        try:
            self.tmp = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={gpu_id(self.index)}", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=self.tmp, stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None
        return self

    def __exit__(self, *exc):
        if self.nvml.ok:
            self.nvml.__exit__(*exc)
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        if self.nvml.ok:
            got = self.nvml.summary()
            if got:
                return got
        if self.proc is None or self.tmp is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no clock samples"]}
        self.tmp.flush()
        rows = []
        with open(self.tmp.name) as f:
            for line in f:
                parts = [p.strip() for p in line.split(",")]
                if len(parts) >= 9:
                    rows.append(parts)
        os.unlink(self.tmp.name)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        smax = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if r[5 + i].lower() == "active"})
        loaded = [v for v in sm if smax and v > 0.5 * max(smax)] or sm
        return {"sm_mhz": statistics.median(loaded) if loaded else None,
                "sm_max_mhz": max(smax) if smax else None, "reasons": reasons, "samples": len(rows)}


def cpu_scalar_baseline(n: int = SCALAR_SAMPLE_N, min_seconds: float = 2.0) -> dict:
    """The reference's scalar path on one core: the sequential rand(double*, n)
    of original/mrg8.cpp:231-239 (ORIGINAL scaling), restated in
    oracle/mrg8_oracle.c (orc_rand_f64); first run discarded, as the
    reference's drivers do."""
    from oracle.pyoracle import Oracle
    o = Oracle()
    st = o.seed(SEED)
    o.rand_f64(st, n, 0)
    runs, t0 = 0, time.perf_counter()
    while True:
        o.rand_f64(st, n, 0)
        runs += 1
        el = time.perf_counter() - t0
        if el >= min_seconds and runs >= 2:
            break
    return {"value": round(n * runs / el / 1e9, 4), "unit": UNIT, "cores": 1, "kind": "port",
            "sample": f"{runs} runs of {n} sequential fp64 ORIGINAL samples (original/mrg8.cpp rand), "
                      "first run discarded"}


def cpu_baseline(n: int, kind: int, min_seconds: float = 3.0):
    """The reference's CPU path on all host cores: the knl/ block-split
    generator (knl/mrg8_vec.h:500-525, its non-AVX A^8 recurrence), restated
    in oracle/mrg8_oracle.c.  Returns (Gsamples/s, cores, sample text)."""
    import numpy as np

    from oracle.pyoracle import KIND_DTYPE, Oracle
    o = Oracle()
    cores = os.cpu_count() or 1
    st = o.seed(SEED)
    out = np.empty(n, dtype=KIND_DTYPE[kind])
    o.generate(st, n, kind, nthreads=cores, out=out)  # first run discarded (page faults)
    runs, t0 = 0, time.perf_counter()
    while True:
        o.generate(st, n, kind, nthreads=cores, out=out)
        runs += 1
        el = time.perf_counter() - t0
        if el >= min_seconds and runs >= 3:
            break
    gs = n * runs / el / 1e9
    return gs, cores, f"{runs} runs of {n} fp64 SHIFTED samples ({n * 8 >> 20} MiB), first run discarded"


def run_batched(dev, steps: int = 5, count: int = 10_000, max_log2: int = 22, seed: int = 4, tune: bool = True):
    """Uneven batch: `count` generators with distinct seeds, lengths log-uniform in
    [1, 2^max_log2], kinds uniform over fp64/fp32/uint32 (SHIFTED uniforms);
    one autotuned graph-captured batch launch vs one bulk launch per instance.
    Both produce the same values (tests/test_batch_gpu.py)."""
    import numpy as np
    import torch

    import mrg8_gb300 as m
    rng = np.random.default_rng(seed)
    kinds = [m.F64_SHIFTED, m.F32_SHIFTED, m.U32]
    lens = np.minimum((2.0 ** rng.uniform(0, max_log2, count)).astype(np.int64), 1 << max_log2)
    ks = rng.integers(0, 3, count)
    dts = {m.F64_SHIFTED: torch.float64, m.F32_SHIFTED: torch.float32, m.U32: torch.int32}
    insts = []
    total = 0
    nbytes = 0
    for i in range(count):
        kind = kinds[int(ks[i])]
        n = int(lens[i])
        out = torch.empty(n, dtype=dts[kind], device=dev)
        insts.append((m.seed_state((i * 2654435761 + 12345) & 0xFFFFFFFF), 0, out, kind))
        total += n
        nbytes += n * out.element_size()
    b = m.Batch(insts)
    tuned = b.autotune() if tune else b.config
    stream = torch.cuda.current_stream(dev)

    def timed(fn, reps):
        fn()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        t0 = time.perf_counter()
        e0.record(stream)
        for _ in range(reps):
            fn()
        e1.record(stream)
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / 1e3 / reps, (time.perf_counter() - t0) / reps

    tb, wb = timed(b.launch, steps)
    te, we = timed(b.launch_each, max(2, steps // 2))
    st = b.stats()
    b.close()
    del insts
    torch.cuda.empty_cache()
    return {"instances": count, "outputs": total, "bytes": nbytes, "tiles": st["tiles"], "config": tuned,
            "batched_gsamples_per_s": round(total / tb / 1e9, 3), "batched_ms": round(tb * 1e3, 3),
            "per_instance_gsamples_per_s": round(total / te / 1e9, 3), "per_instance_ms": round(te * 1e3, 3),
            "per_instance_wall_ms": round(we * 1e3, 3), "speedup": round(te / tb, 2),
            "lengths": f"log-uniform in [1, 2^{max_log2}]", "kinds": "fp64/fp32/u32 uniform (SHIFTED)"}


def run_jumps(dev, reps: int = 5, count: int = 65_536, n: int = 4096, seed: int = 20240331) -> dict:
    """Config 3: 65,536 substreams of seed 13579, each jumped by an offset drawn
    uniformly in [0, 2^63), with 4,096 uint32 outputs each (2^28 outputs,
    1 GiB): the device jumps alone (mrg8g_jump_states, one warp per offset)
    and the whole workload as one batch launch (a jump per tile, then the
    outputs).  Both are checked bit for bit in tests/test_batch_gpu.py."""
    import numpy as np
    import torch

    import mrg8_gb300 as m
    rng = np.random.default_rng(seed)
    st = m.seed_state(SEED)
    offs = rng.integers(0, 2**63, count, dtype=np.int64)
    d_off = torch.from_numpy(offs).to(dev)
    out = torch.empty((count, n), dtype=torch.int32, device=dev)
    b = m.Batch([(st, int(offs[i]), out[i], m.U32) for i in range(count)])
    stream = torch.cuda.current_stream(dev)

    def timed(fn):
        for _ in range(2):
            fn()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(reps):
            fn()
        e1.record(stream)
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / 1e3 / reps

    tj = timed(lambda: m.jump_states(st, d_off))
    tb = timed(b.launch)
    b.close()
    del out
    torch.cuda.empty_cache()
    return {"substreams": count, "outputs_each": n, "offsets": "uniform in [0, 2^63)",
            "jumps_per_s": round(count / tj, 1), "jump_ms": round(tj * 1e3, 4),
            "batch_ms": round(tb * 1e3, 4), "batch_gsamples_per_s": round(count * n / tb / 1e9, 3)}


def _served_row(r: dict, rate: float, seconds: float) -> dict:
    return {"rate_per_s": rate, "duration_s": seconds, "requests": r["requests"],
            "gsamples_per_s": round(r["gsamples_per_s"], 3), "p50_us": round(r["p50_us"], 1),
            "p90_us": round(r["p90_us"], 1), "p99_us": round(r["p99_us"], 1), "max_us": round(r["max_us"], 1),
            "mean_batch": round(r["mean_batch"], 2), "launches": r["launches"], "max_inflight": r["max_inflight"],
            "overlapped_launches": r["overlapped_launches"], "mean_kernel_us": round(r["mean_kernel_us"], 2),
            "peak_bytes": r["peak_bytes"],
            "late_submits": r["late_submits"]}


def run_served(seconds: float, rate: float = 20_000.0, sweep=(20_000.0, 50_000.0, 100_000.0, 200_000.0),
               sweep_seconds: float = 2.0):
    """Serving load (config 5): Poisson arrivals at `rate`/s for `seconds`,
    offsets uniform in [0, 2^48), lengths log-uniform in [2^8, 2^26], kinds
    fp64/fp32/uint32, 16 GiB admission budget, results released on completion;
    then the same load for `sweep_seconds` at each rate of `sweep`, to show
    where latency or delivered throughput stops following the offered load."""
    from mrg8_gb300.serve import Server
    kw = dict(n_min=1 << 8, n_max=1 << 26, offset_max=1 << 48, kinds_mask=0b10101)
    with Server(budget_bytes=16 << 30) as srv:
        srv.loadtest(rate=rate, duration_s=min(1.0, seconds), rng_seed=7, **kw)  # warm-up
        r = srv.loadtest(rate=rate, duration_s=seconds, rng_seed=11, **kw)
        rows = [_served_row(srv.loadtest(rate=q, duration_s=sweep_seconds, rng_seed=13 + i, **kw), q, sweep_seconds)
                for i, q in enumerate(sweep)]
    out = _served_row(r, rate, seconds)
    out["budget_bytes"] = 16 << 30
    out["offered_gsamples_per_s"] = round(rate * 5.39e6 / 1e9, 1)
    out["rate_sweep"] = rows
    return out


def run_reference(args) -> None:
    ws, rank, _ = dist_env()
    if rank != 0:
        return
    import numpy as np

    from oracle.pyoracle import F64_SHIFTED, REF_DIR, KIND_DTYPE, Oracle, reference_dir
    cores = os.cpu_count() or 1
    kind_name, impl = "port", None
    refdir = reference_dir()
    if os.path.exists(os.path.join(REF_DIR, "libmrg8_ref_knl.so")) and refdir is not None:
        try:
            from oracle.pyoracle import RefLib
            impl = RefLib("knl", refdir)
            kind_name = "reference"
        except OSError:
            impl = None
    o = Oracle()
    st = o.seed(SEED)
    n = args.n
    out = np.empty(n, dtype=KIND_DTYPE[F64_SHIFTED])

    def step():
        if impl is not None:
            impl.rand_tp(st, n, cores)
        else:
            o.generate(st, n, F64_SHIFTED, nthreads=cores, out=out)

    for _ in range(args.warmup):
        step()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        step()
    el = time.perf_counter() - t0
    value = n * args.steps / el / 1e9
    sample = (f"each step {n} fp64 SHIFTED samples of the same stream (seed {SEED}), "
              + ("knl/mrg8.h rand_tp compiled from the reference" if impl is not None else
                 "oracle port of knl/mrg8_vec.h mrg8_vec_outer_tp (block split + A^8 recurrence)")
              + f", {cores} threads")
    scalar = None if args.skip_cpu else cpu_scalar_baseline(min(SCALAR_SAMPLE_N, n))
    ref_gpu = None if args.skip_ref_gpu else reference_gpu_kernel()
    line = {"impl": "reference", "metric": METRIC, "value": round(value, 4), "unit": UNIT, "n_gpus": ws,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(el / args.steps * 1e3, 3),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic", "config": workload_config(n, ws),
            "cpu_baseline": {"value": round(value, 4), "unit": UNIT, "cores": cores, "kind": kind_name,
                             "sample": sample, "scalar_original": scalar},
            "e2e": {"value": round(value, 4), "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "ref_gpu": ref_gpu}
    print(json.dumps(line), flush=True)


def reference_gpu_kernel() -> dict | None:
    """The reference's own GPU kernel, rng_outer_32 (cuda/mrg8_cuda.cu:282-399),
    compiled from its sources into oracle/_ref/mrg8_ref_cuda.cubin: checked
    bit for bit against the oracle at 2^24 and timed (kernel only, CUDA
    events) at 2^30 over the launch shapes its own driver sweeps
    (cuda/tests/test_mrg8_outer.cu:50-76), with the SM clocks sampled
    meanwhile.  None where the cubin was not built."""
    try:
        import torch
        if not torch.cuda.is_available():
            return None
    except ImportError:
        return None
    from oracle import ref_gpu_run as rg
    if not rg.available():
        return {"unavailable": "the reference's sources were not present where this tree was built"}
    rg.build_driver()
    chk = rg.check(1 << 24)
    shapes = [(t, b) for t in (64 * 1024, 256 * 1024, 1024 * 1024) for b in (32, 64, 128, 256, 512)]
    with ClockSampler(0) as clk:
        rows = rg.time_shapes(1 << 30, 10, shapes)
    best = max(rows, key=lambda r: r["gsamples_per_s"])
    default = next(r for r in rows if r["tnum"] == 64 * 1024 and r["bs"] == 64)
    return {"kernel": "rng_outer_32 (cuda/mrg8_cuda.cu:282-399), built from the reference sources for sm_103a",
            "n": 1 << 30, "dtype": "f64 SHIFTED", "mismatches": chk["mismatches"], "checked_outputs": chk["n"],
            "next_state_equal": chk["next_state_equal"], "default_shape": default, "best_shape": best,
            "unit": UNIT, "timing": "kernel only, CUDA events, 10 launches per shape", "clocks": clk.summary()}


def run_ceilings(args) -> None:
    """Denominators beside the measured copy peak: the write-only HBM rate
    (memset and fill of 8 GiB, the bulk kernel's traffic pattern being pure
    writes) and the host link (1 GiB to and from pinned host memory, the
    bound of the e2e figure).  CUDA events on the current stream, best of
    `args.steps` after `args.warmup` untimed runs; SM clocks sampled."""
    import torch
    dev = torch.device("cuda", 0)
    torch.cuda.set_device(dev)
    stream = torch.cuda.current_stream(dev)
    buf = torch.empty(1 << 30, dtype=torch.float64, device=dev)
    host = torch.empty(1 << 27, dtype=torch.float64, pin_memory=True)
    dsmall = buf[: 1 << 27]

    def best(fn, nbytes):
        for _ in range(max(args.warmup, 1)):
            fn()
        torch.cuda.synchronize()
        ts = []
        for _ in range(max(args.steps, 3)):
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(stream)
            fn()
            b.record(stream)
            b.synchronize()
            ts.append(a.elapsed_time(b) / 1e3)
        return {"gbs": round(nbytes / min(ts) / 1e9, 1), "bytes": nbytes, "best_ms": round(min(ts) * 1e3, 4),
                "median_ms": round(statistics.median(ts) * 1e3, 4)}

    with ClockSampler(0) as clk:
        out = {"memset_8GiB": best(lambda: buf.zero_(), buf.numel() * 8),
               "fill_8GiB": best(lambda: buf.fill_(0.5), buf.numel() * 8),
               "d2h_pinned_1GiB": best(lambda: host.copy_(dsmall, non_blocking=True), host.numel() * 8),
               "h2d_pinned_1GiB": best(lambda: dsmall.copy_(host, non_blocking=True), host.numel() * 8)}
    peaks, src = measured_peaks()
    print(json.dumps({"ceilings": out, "copy_peak_gbs": peaks.get("hbm_gbs"), "copy_peak_source": src,
                      "clocks": clk.summary(), "steps": max(args.steps, 3), "warmup": max(args.warmup, 1)}),
          flush=True)


def run_gpu(args) -> None:
    import numpy as np
    import torch

    import mrg8_gb300 as m
    ws, rank, local = dist_env()
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    pg = None
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=dev)
        pg = dist
    n = args.n
    kind = m.F64_SHIFTED
    g = m.MRG8(SEED)
    if rank:
        g.jump_ahead(rank * n)           # this rank's shard of the one stream
    st0 = g.get_state()
    out = torch.empty(n, dtype=torch.float64, device=dev)
    stream = torch.cuda.current_stream(dev)

    def step():
        g.set_state(st0)
        g.rand(out, scaling=1)

    for _ in range(max(args.warmup, 0)):
        step()
    torch.cuda.synchronize()
    if pg:
        pg.barrier()
    evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    with ClockSampler(local) as clk:
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for i in range(args.steps):
            evs[i][0].record(stream)
            step()
            evs[i][1].record(stream)
        torch.cuda.synchronize()
        wall = time.perf_counter() - t0
    if pg:
        pg.barrier()
    per = [a.elapsed_time(b) for a, b in evs]          # ms, one launch per step
    total_ms = sum(per)
    if pg:
        t = torch.tensor([total_ms, wall * 1e3], device=dev, dtype=torch.float64)
        pg.all_reduce(t, op=pg.ReduceOp.MAX)
        total_ms = float(t[0])
    value = ws * n * args.steps / (total_ms / 1e3) / 1e9
    peaks, peak_src = measured_peaks()
    avg_launch_s = statistics.mean(per) / 1e3
    achieved = 8.0 * n / avg_launch_s / 1e9
    hbm = float(peaks.get("hbm_gbs", 6800.0))

    # fp32 at the same size (secondary line item; not the headline).
    f32 = None
    if not args.skip_f32:
        out32 = torch.empty(n, dtype=torch.float32, device=dev)
        for _ in range(3):
            g.set_state(st0)
            g.rand_f32(out32, scaling=1)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        reps = max(3, args.steps // 2)
        e0.record(stream)
        for _ in range(reps):
            g.set_state(st0)
            g.rand_f32(out32, scaling=1)
        e1.record(stream)
        torch.cuda.synchronize()
        f32_s = e0.elapsed_time(e1) / 1e3 / reps
        del out32
        f32 = {"value": round(n / f32_s / 1e9, 4), "unit": UNIT, "gbs": round(4.0 * n / f32_s / 1e9, 1),
               "frac_hbm": round(4.0 * n / f32_s / 1e9 / hbm, 4)}
        # The remaining output kinds at the same size (line items).
        from mrg8_gb300 import _lib as L
        buf = torch.empty(n * 8, dtype=torch.uint8, device=dev)
        f32["other_kinds"] = {}
        for name, kd, dt, eb in (("u32", L.U32, torch.int32, 4), ("f64_original", L.F64_ORIGINAL, torch.float64, 8),
                                 ("f32_original", L.F32_ORIGINAL, torch.float32, 4)):
            view = buf.view(dt)[:n]
            for _ in range(3):
                g.set_state(st0)
                g._generate(view, n, kd)
            e0.record(stream)
            for _ in range(reps):
                g.set_state(st0)
                g._generate(view, n, kd)
            e1.record(stream)
            torch.cuda.synchronize()
            ks = e0.elapsed_time(e1) / 1e3 / reps
            f32["other_kinds"][name] = {"value": round(n / ks / 1e9, 4), "gbs": round(eb * n / ks / 1e9, 1),
                                        "frac_hbm": round(eb * n / ks / 1e9 / hbm, 4)}
        del buf

    # End to end through the C ABI with a pinned host buffer.
    e2e = None
    if not args.skip_e2e:
        host = torch.empty(n, dtype=torch.float64, pin_memory=True)
        hp = host.numpy()
        for _ in range(2):
            g.set_state(st0)
            g._generate(hp, n, kind)
        if pg:
            pg.barrier()
        esteps = max(3, min(args.steps, 5))
        t0 = time.perf_counter()
        for _ in range(esteps):
            g.set_state(st0)
            g._generate(hp, n, kind)
        el = time.perf_counter() - t0
        if pg:
            t = torch.tensor([el], device=dev, dtype=torch.float64)
            pg.all_reduce(t, op=pg.ReduceOp.MAX)
            el = float(t[0])
        e2e = {"value": round(ws * n * esteps / el / 1e9, 4), "unit": UNIT, "h2d_bytes_per_step": 32,
               "d2h_bytes_per_step": 8 * n, "steps": esteps,
               "path": "mrg8g_generate_host (C ABI) into pinned host memory; the 32-byte state travels as a "
                       "kernel argument"}
        del host

    batched = None if args.skip_batch or rank else run_batched(dev, count=args.batch_count, tune=not args.batch_no_tune)
    jumps = None if args.skip_batch or rank else run_jumps(dev)
    served = None if args.skip_serve or rank else run_served(args.serve_seconds)

    # Spot check of this run's output against the oracle (first 2^20 values).
    from oracle.pyoracle import F64_SHIFTED as O_F64S, Oracle
    chk = min(n, 1 << 20)
    ref, _ = Oracle().generate(st0, chk, O_F64S, nthreads=os.cpu_count() or 8)
    ok = bool(np.array_equal(out[:chk].cpu().numpy().view(np.uint64), ref.view(np.uint64)))

    if rank != 0:
        if pg:
            pg.destroy_process_group()
        return
    cpu = None
    if not args.skip_cpu:
        v, cores, sample = cpu_baseline(CPU_SAMPLE_N, O_F64S)
        cpu = {"value": round(v, 4), "unit": UNIT, "cores": cores, "kind": "port", "sample": sample,
               "scalar_original": cpu_scalar_baseline()}
    traffic = profiled_traffic("k_plain_f64_2p30.md")
    line = {
        "metric": METRIC, "value": round(value, 4), "unit": UNIT, "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(total_ms / args.steps, 4), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": workload_config(n, ws),
        "layout": "1 warp tile per resident warp, 2 substreams per lane",
        "roofline": {"bound": "hbm", "achieved": round(achieved, 1), "peak": hbm, "unit": "GB/s",
                     "frac": round(achieved / hbm, 4), "peak_source": f"{peak_src} hbm_gbs (copy)",
                     "traffic": traffic, "algorithmic_bytes_per_launch": 8 * n},
        "f32": f32,
        "e2e": e2e, "cpu_baseline": cpu, "batched": batched, "jump_stress": jumps, "served": served,
        "clocks": clk.summary(), "gpu_launches": args.steps,
        "parity_spot_check": ok, "wall_s": round(wall, 4),
    }
    print(json.dumps(line), flush=True)
    if pg:
        pg.destroy_process_group()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--ceilings", action="store_true", help="measure the write-only HBM and host-link ceilings")
    ap.add_argument("--skip-e2e", action="store_true")
    ap.add_argument("--skip-cpu", action="store_true")
    ap.add_argument("--skip-f32", action="store_true")
    ap.add_argument("--skip-batch", action="store_true")
    ap.add_argument("--skip-serve", action="store_true")
    ap.add_argument("--serve-seconds", type=float, default=60.0)
    ap.add_argument("--skip-ref-gpu", action="store_true", help="reference arm without its GPU-kernel leg")
    ap.add_argument("--batch-count", type=int, default=10_000, help="instances of the batched leg (profiling)")
    ap.add_argument("--batch-no-tune", action="store_true", help="batched leg with the default config (profiling)")
    ap.add_argument("--n", type=int, default=N_PER_RANK, help="outputs per GPU (profiling of small cases)")
    args = ap.parse_args()
    if args.ceilings:
        run_ceilings(args)
    elif args.impl == "reference":
        run_reference(args)
    else:
        run_gpu(args)


if __name__ == "__main__":
    main()
