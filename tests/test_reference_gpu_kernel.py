"""The reference's own GPU kernel (rng_outer_32 of cuda/mrg8_cuda.cu) on this
GPU, where its cubin was built (oracle/_ref/, from the reference sources):
its output for seed 13579 equals the oracle's SHIFTED fp64 stream and ours,
bit for bit.  Skipped where the cubin is absent."""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_reference_kernel_equals_oracle_and_ours(cuda):
    from oracle import ref_gpu_run as rg
    if not rg.available():
        pytest.skip("reference cubin not built here (no reference sources)")
    rg.build_driver()
    n = 1 << 22
    res = rg.check(n)
    assert res["mismatches"] == 0 and res["next_state_equal"], res
    import torch

    import mrg8_gb300 as m
    g = m.MRG8Cuda(rg.SEED)
    ours = torch.empty(n, dtype=torch.float64, device=cuda)
    g.mrg8_outer_32(ours, n)
    torch.cuda.synchronize()
    from oracle.pyoracle import F64_SHIFTED, Oracle
    o = Oracle()
    want, _ = o.generate(o.seed(rg.SEED), n, F64_SHIFTED, nthreads=os.cpu_count() or 4)
    assert np.array_equal(ours.cpu().numpy().view(np.uint64), want.view(np.uint64))
