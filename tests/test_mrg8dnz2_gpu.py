"""mrg8dnz2 through the Python mirror of the reference class, against the
oracle's restatement of the reference's ring-buffer generator: ORIGINAL
scaling as cuda/mrg8.cpp:290-339 (the default) and SHIFTED as
knl/mrg8.h:387-436 (scaling=1), on consecutive calls of sizes around the
reference's 1024-deep buffer, into device tensors and host arrays."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

SIZES = (1, 1023, 1024, 1025, 3000, 1000000)


@pytest.mark.parametrize("scaling", [0, 1])
@pytest.mark.parametrize("where", ["device", "host"])
def test_mrg8dnz2_matches_the_oracle(cuda, oracle, scaling, where):
    import torch

    import mrg8_gb300 as m
    g = m.MRG8(13579)
    st = oracle.seed(13579)
    assert np.array_equal(g.get_state(), st)
    for n in SIZES:
        if where == "device":
            buf = torch.empty(n, dtype=torch.float64, device=cuda)
            g.mrg8dnz2(buf, scaling=scaling) if scaling else g.mrg8dnz2(buf)
            got = buf.cpu().numpy()
        else:
            got = np.empty(n, dtype=np.float64)
            g.mrg8dnz2(got, scaling=scaling) if scaling else g.mrg8dnz2(got)
        want, st = oracle.mrg8dnz2(st, n, scaling)
        assert np.array_equal(got.view(np.uint64), want.view(np.uint64)), (n, scaling, where)
        assert np.array_equal(g.get_state(), st), (n, scaling, where)
