"""The allocation-free batch entry point, mrg8g_batch_generate_noalloc.

It serves callers that may not allocate device memory themselves (a host
application or framework allocator owns the GPU's memory, or a latency-critical
loop cannot take cudaMalloc's synchronisation): its scratch is a fixed array
inside the library.  This file is collected last so that a failure here comes
after every other test has run; it also passes on its own in a fresh process.
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
        for k, ((buf, v), w) in enumerate(zip(outs, want)):
            assert np.array_equal(v.cpu().numpy().view(np.uint8), w), (call, k)
            lead = buf.numel() - v.numel()
            assert bool((buf[:lead] == 0).all()), (call, k)


def test_no_alloc_rejects_oversized_batches(cuda):
    import mrg8_gb300 as m
    from mrg8_gb300 import _lib as L
    lib = m.load()
    arr = (L.Instance * (L_MAX + 1))()
    assert lib.mrg8g_batch_generate_noalloc(arr, L_MAX + 1, None) == L.ERR_BUDGET
    assert b"no-alloc limit" in lib.mrg8g_last_error()


L_MAX = 4096  # MRG8G_NOALLOC_MAX_INSTANCES of include/mrg8g.h
