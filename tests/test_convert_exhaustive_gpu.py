"""The uniform conversion as compiled for the GPU (integer-only for fp64, on the
FP32 pipes for fp32), on every stream value: all S in [1, 2^31 - 1] go through the device conversion (the same
device functions the generators use) in both scalings, fp64 and fp32, and
must equal IEEE round-to-nearest of (S - shift) * (1.0 / (2^31 - 1)) computed
with the GPU's own fp64 multiply, bit for bit."""
import pytest

pytestmark = pytest.mark.gpu

P = 2147483647
CHUNK = 1 << 28


def test_every_stream_value_both_scalings(cuda):
    import torch

    import mrg8_gb300 as m
    rnorm = 1.0 / P
    s = torch.empty(CHUNK, dtype=torch.int64, device=cuda)
    o64 = torch.empty(CHUNK, dtype=torch.float64, device=cuda)
    o32 = torch.empty(CHUNK, dtype=torch.float32, device=cuda)
    for start in range(1, P + 1, CHUNK):
        n = min(CHUNK, P + 1 - start)
        torch.arange(start, start + n, dtype=torch.int64, device=cuda, out=s[:n])
        raw = s[:n].to(torch.int32)
        for shift in (0, 1):  # ORIGINAL S * rnorm, SHIFTED (S - 1) * rnorm
            m.convert(raw, o64[:n], shift)
            m.convert(raw, o32[:n], shift)
            want = (s[:n] - shift).to(torch.float64) * rnorm
            bad64 = int((o64[:n].view(torch.int64) != want.view(torch.int64)).sum())
            bad32 = int((o32[:n].view(torch.int32) != want.to(torch.float32).view(torch.int32)).sum())
            assert bad64 == 0 and bad32 == 0, (start, shift, bad64, bad32)
    torch.cuda.synchronize()
