"""Concurrent use from several host threads: each thread owns a generator
handle and a CUDA stream and generates device and host outputs at the same
time as the others; every result equals its own stream segment in the
oracle.  (The reference's class is not thread-safe; this library's per-device
set-up is guarded and its handles hold no shared mutable state.)"""
import threading

import numpy as np
import pytest

from oracle import pyoracle as po

pytestmark = pytest.mark.gpu


def test_threads_with_own_handles_and_streams(cuda, oracle):
    import torch

    import mrg8_gb300 as m
    nthreads, rounds = 6, 4
    sizes = [1, 777, 1 << 16, (1 << 20) + 3]
    results, errors = {}, []

    def work(t):
        try:
            g = m.MRG8(1000 + t)
            s = torch.cuda.Stream()
            outs = []
            with torch.cuda.stream(s):
                for r in range(rounds):
                    n = sizes[(t + r) % len(sizes)]
                    d = torch.empty(n, dtype=torch.float64 if r % 2 else torch.float32, device=cuda)
                    if r % 2:
                        g.rand(d, scaling=1)
                    else:
                        g.rand_f32(d, scaling=0)
                    h = np.empty(n, dtype=np.uint32)
                    g.randint(h)                    # host buffer path between device calls
                    outs.append((d, h))
            s.synchronize()
            results[t] = [(d.cpu().numpy(), h) for d, h in outs]
        except Exception as e:  # reported below
            errors.append((t, repr(e)))

    ths = [threading.Thread(target=work, args=(t,)) for t in range(nthreads)]
    for th in ths:
        th.start()
    for th in ths:
        th.join()
    assert not errors, errors
    for t in range(nthreads):
        st = oracle.seed(1000 + t)
        for r, (d, h) in enumerate(results[t]):
            n = sizes[(t + r) % len(sizes)]
            kind = po.F64_SHIFTED if r % 2 else po.F32_ORIGINAL
            want, st = oracle.generate(st, n, kind)
            assert np.array_equal(d.view(np.uint8), want.view(np.uint8)), (t, r)
            want_u, st = oracle.generate(st, n, po.U32)
            assert np.array_equal(h, want_u), (t, r)
