"""The allocation-free batch entry point, mrg8g_batch_generate_noalloc.

It serves callers that may not allocate device memory themselves (a host
application or framework allocator owns the GPU's memory, or a latency-critical
loop cannot take cudaMalloc's synchronisation): its scratch is a fixed array
inside the library.  Its outputs are checked against the existing batch entry
point and against the oracle, on two calls in a row; its limits and its refusal
of a capturing stream are checked too.  This file is collected last so that a
failure here comes after every other test has run; it also passes on its own in
a fresh process.
"""
import ctypes as C

import numpy as np
import pytest

from oracle import pyoracle as po

pytestmark = pytest.mark.gpu

KINDS = [po.U32, po.F64_ORIGINAL, po.F64_SHIFTED, po.F32_ORIGINAL, po.F32_SHIFTED]


def make(cuda, rng, count):
    import torch

    import mrg8_gb300 as m
    from mrg8_gb300 import _lib as L
    dts = {po.U32: torch.int32, po.F64_ORIGINAL: torch.float64, po.F64_SHIFTED: torch.float64,
           po.F32_ORIGINAL: torch.float32, po.F32_SHIFTED: torch.float32}
    insts, outs = [], []
    for i in range(count):
        kind = KINDS[int(rng.integers(0, 5))]
        n = int(2 ** rng.uniform(0, 17)) if i % 9 else int(rng.integers(0, 9))
        lead = int(rng.integers(0, 4))
        buf = torch.zeros(n + lead, dtype=dts[kind], device=cuda)
        view = buf[lead:]
        inst = L.Instance()
        inst.state[:] = [int(v) for v in m.seed_state(int(rng.integers(0, 2**32)))]
        inst.offset = int(rng.integers(0, 2**62)) if i % 4 == 0 else 0
        inst.n, inst.out, inst.kind, inst.reserved = n, view.data_ptr() if n else 0, kind, 0
        insts.append(inst)
        outs.append((buf, view))
    return (L.Instance * len(insts))(*insts), outs


def reference_outputs(lib, arr, count, outs, stream):
    """The existing entry point (batch plan + launch) on copies of the buffers."""
    import torch
    saved = [v.clone() for _, v in outs]
    plan = C.c_void_p()
    assert lib.mrg8g_batch_create(arr, count, None, C.byref(plan)) == 0
    assert lib.mrg8g_batch_launch(plan, C.c_void_p(stream)) == 0
    torch.cuda.synchronize()
    want = [v.cpu().numpy().view(np.uint8).copy() for _, v in outs]
    lib.mrg8g_batch_destroy(plan)
    for (_, v), s in zip(outs, saved):
        v.copy_(s)
    return want


def test_no_alloc_matches_the_batch_path_on_two_calls_in_a_row(cuda):
    import torch

    import mrg8_gb300 as m
    lib = m.load()
    stream = torch.cuda.current_stream().cuda_stream
    rng = np.random.default_rng(77)
    for call in range(2):
        arr, outs = make(cuda, rng, 150 + 50 * call)
        want = reference_outputs(lib, arr, len(outs), outs, stream)
        for _, v in outs:
            v.zero_()
        rc = lib.mrg8g_batch_generate_noalloc(arr, len(outs), C.c_void_p(stream))
        assert rc == 0, lib.mrg8g_last_error()
        torch.cuda.synchronize()
        o = po.Oracle()
        for k, ((buf, v), w) in enumerate(zip(outs, want)):
            got = v.cpu().numpy().view(np.uint8)
            assert np.array_equal(got, w), (call, k)
            lead = buf.numel() - v.numel()
            assert bool((buf[:lead] == 0).all()), (call, k)
            inst = arr[k]
            if inst.n:
                st = o.jump(np.array(inst.state, dtype=np.uint32), int(inst.offset))
                ref, _ = o.generate(st, int(inst.n), int(inst.kind))
                assert np.array_equal(got, ref.view(np.uint8)), ("oracle", call, k)


def test_no_alloc_rejects_oversized_batches(cuda):
    import mrg8_gb300 as m
    from mrg8_gb300 import _lib as L
    lib = m.load()
    arr = (L.Instance * (L_MAX + 1))()
    assert lib.mrg8g_batch_generate_noalloc(arr, L_MAX + 1, None) == L.ERR_BUDGET
    assert b"no-alloc limit" in lib.mrg8g_last_error()


def test_no_alloc_rejects_more_tiles_than_its_limit(cuda):
    """Two instances of 1.5 * 2^30 outputs need 98,304 body tiles of 32,768
    outputs, above the 65,536 the scratch array holds: refused before anything
    is enqueued.  Both point at one buffer large enough for either instance,
    so not even a wrongly accepted call could write out of bounds."""
    import torch

    import mrg8_gb300 as m
    from mrg8_gb300 import _lib as L
    lib = m.load()
    n = 3 << 29
    buf = torch.empty(n, dtype=torch.int32, device=cuda)
    insts = []
    for seed in (1, 2):
        inst = L.Instance()
        inst.state[:] = [int(v) for v in m.seed_state(seed)]
        inst.offset, inst.n, inst.out, inst.kind, inst.reserved = 0, n, buf.data_ptr(), L.U32, 0
        insts.append(inst)
    arr = (L.Instance * 2)(*insts)
    stream = torch.cuda.current_stream().cuda_stream
    assert lib.mrg8g_batch_generate_noalloc(arr, 2, C.c_void_p(stream)) == L.ERR_BUDGET
    assert b"no-alloc limit" in lib.mrg8g_last_error()
    del buf


def test_no_alloc_refuses_a_capturing_stream(cuda):
    """Its descriptors come from a host staging area that every call rewrites,
    so a call on a stream under capture is refused and enqueues nothing."""
    import torch

    import mrg8_gb300 as m
    from mrg8_gb300 import _lib as L
    lib = m.load()
    assert lib.mrg8g_batch_generate_noalloc(None, 0, None) == 0  # per-device set-up, outside the capture
    rng = np.random.default_rng(5)
    arr, outs = make(cuda, rng, 8)
    side = torch.cuda.Stream()
    x = torch.zeros(4, device=cuda)
    g = torch.cuda.CUDAGraph()
    torch.cuda.synchronize()
    with torch.cuda.stream(side):
        g.capture_begin()
        x.add_(1)
        rc = lib.mrg8g_batch_generate_noalloc(arr, len(outs), C.c_void_p(side.cuda_stream))
        g.capture_end()
    torch.cuda.synchronize()
    assert rc == L.ERR_INVALID_ARGUMENT
    assert b"capturing" in lib.mrg8g_last_error()
    for buf, _ in outs:
        assert bool((buf == 0).all())


L_MAX = 4096  # MRG8G_NOALLOC_MAX_INSTANCES of include/mrg8g.h
