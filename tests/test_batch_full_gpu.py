"""Config 4 at its full size, checked output by output: the 10,000 uneven
instances of bench.py's batched leg (distinct seeds, lengths log-uniform in
[1, 2^22], kinds uniform over fp64 / fp32 / uint32 SHIFTED; 2.76e9 outputs,
14.7 GB) in one graph-captured batch launch with the autotuned shape, every
instance against the oracle's restatement of its own sequential stream."""
import concurrent.futures as cf
import os

import numpy as np
import pytest

from oracle import pyoracle as po

pytestmark = pytest.mark.gpu


def test_ten_thousand_instances_bit_exact(cuda, oracle):
    import torch

    import mrg8_gb300 as m
    count, max_log2 = 10_000, 22
    rng = np.random.default_rng(4)                       # the plan of bench.py's batched leg
    kinds = [m.F64_SHIFTED, m.F32_SHIFTED, m.U32]
    lens = np.minimum((2.0 ** rng.uniform(0, max_log2, count)).astype(np.int64), 1 << max_log2)
    ks = rng.integers(0, 3, count)
    dts = {m.F64_SHIFTED: torch.float64, m.F32_SHIFTED: torch.float32, m.U32: torch.int32}
    odk = {m.F64_SHIFTED: po.F64_SHIFTED, m.F32_SHIFTED: po.F32_SHIFTED, m.U32: po.U32}
    # One buffer per kind; instance outputs are consecutive slices of it.
    total = {k: int(sum(int(lens[i]) for i in range(count) if kinds[int(ks[i])] == k)) for k in kinds}
    bufs = {k: torch.empty(total[k], dtype=dts[k], device=cuda) for k in kinds}
    pos = {k: 0 for k in kinds}
    insts, plan = [], []
    for i in range(count):
        k = kinds[int(ks[i])]
        n = int(lens[i])
        state = m.seed_state((i * 2654435761 + 12345) & 0xFFFFFFFF)
        insts.append((state, 0, bufs[k][pos[k]:pos[k] + n], k))
        plan.append((state, k, pos[k], n))
        pos[k] += n
    b = m.Batch(insts)
    b.autotune()
    for k in kinds:
        bufs[k].zero_()
    b.launch()
    torch.cuda.synchronize()
    host = {k: bufs[k].cpu().numpy() for k in kinds}
    b.close()

    def check(item):
        state, k, p, n = item
        want, _ = oracle.generate(state, n, odk[k])
        got = host[k][p:p + n]
        return bool(np.array_equal(got.view(np.uint8), want.view(np.uint8)))

    with cf.ThreadPoolExecutor(max_workers=os.cpu_count() or 8) as ex:
        ok = list(ex.map(check, plan, chunksize=64))
    bad = [i for i, v in enumerate(ok) if not v]
    assert not bad, f"{len(bad)} instances differ, first {bad[:5]}"
    assert sum(n for _, _, _, n in plan) == sum(total.values()) > 2.7e9
