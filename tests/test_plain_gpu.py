"""Parity of the sm_103a bulk kernel with the oracle (bit-exact), through the
C ABI (ctypes) and the Python mirror of the reference classes."""
import hashlib

import numpy as np
import pytest

from mrg8_helpers import P, bits64, state_with_output, u32_view
from oracle import pyoracle as po

pytestmark = pytest.mark.gpu

KINDS = [po.U32, po.F64_ORIGINAL, po.F64_SHIFTED, po.F32_ORIGINAL, po.F32_SHIFTED]


def torch_dtype(kind):
    import torch
    return {po.U32: torch.int32, po.F64_ORIGINAL: torch.float64, po.F64_SHIFTED: torch.float64,
            po.F32_ORIGINAL: torch.float32, po.F32_SHIFTED: torch.float32}[kind]


def as_bytes(x):
    if hasattr(x, "detach"):
        x = x.detach().cpu().numpy()
    return np.ascontiguousarray(x).view(np.uint8)


def sha(a):
    return hashlib.sha256(as_bytes(a).tobytes()).hexdigest()


def gen_device(g, n, kind, cuda, offset=0, canary=True):
    """Generate n outputs of `kind` into a device buffer at element `offset`."""
    import torch
    dt = torch_dtype(kind)
    buf = torch.full((n + offset + 5,), -7, dtype=dt, device=cuda) if canary else \
        torch.empty(n + offset, dtype=dt, device=cuda)
    g._generate(buf[offset:offset + n], n, kind)
    torch.cuda.synchronize()
    if canary:
        host = buf.cpu()
        ref = torch.full((1,), -7, dtype=dt)
        assert bool((host[:offset] == ref).all()) and bool((host[offset + n:] == ref).all()), "wrote outside"
        return host[offset:offset + n]
    return buf[offset:offset + n].cpu()


def test_seed13579_2p24_known_answers(cuda, kat):
    """Plain single stream, seed 13579, 2^24: fp64 rand + the same positions as
    uint32, bit-exact with original/mrg8.cpp (golden digests)."""
    import mrg8_gb300 as m
    import torch
    k = kat["seed13579"]
    n = 1 << 24
    g = m.MRG8(13579)
    f = torch.empty(n, dtype=torch.float64, device=cuda)
    g.rand(f)                                  # ORIGINAL, as original/mrg8.cpp
    assert g.get_state().tolist() == k["state_after_2^24"]
    g.seed_init(13579)
    r = torch.empty(n, dtype=torch.int32, device=cuda)
    g.randint(r)
    torch.cuda.synchronize()
    assert sha(f) == k["sha256_rand_original_2^24"]
    ints = u32_view(r)
    assert sha(ints) == k["sha256_randint_2^24"]
    assert ints[:64].tolist() == k["randint_first64"]
    assert int(ints.min()) == k["min_2^24"] and int(ints.max()) == k["max_2^24"]
    cg = m.MRG8Cuda(13579)
    cg.mrg8_outer_32(f, n)                     # SHIFTED, as cuda/mrg8_cuda.cu
    torch.cuda.synchronize()
    assert sha(f) == k["sha256_rand_shifted_2^24"]
    cg.seed_init(13579)
    cg.mrg8_inner(f, n, 1024)
    torch.cuda.synchronize()
    assert sha(f) == k["sha256_rand_shifted_2^24"]
    x = torch.empty(n, dtype=torch.float32, device=cuda)
    for sc, key in ((0, "sha256_f32_original_2^24"), (1, "sha256_f32_shifted_2^24")):
        g.seed_init(13579)
        g.rand_f32(x, scaling=sc)
        torch.cuda.synchronize()
        assert sha(x) == k[key]


SIZES = [1, 2, 3, 4, 5, 7, 8, 9, 31, 32, 33, 63, 64, 65, 127, 128, 129, 255, 256, 257, 511, 512, 513,
         1023, 1024, 1025, 4095, 4096, 4097, 65537, 262147, 1000003]


@pytest.mark.parametrize("kind", KINDS)
def test_sizes_and_alignment(cuda, oracle, kind):
    import mrg8_gb300 as m
    g = m.MRG8(2024 + kind)
    rng = np.random.default_rng(kind)
    for n in SIZES:
        offset = int(rng.integers(0, 4))
        st = g.get_state()
        ref, end = oracle.generate(st, n, kind, nthreads=4)
        out = gen_device(g, n, kind, cuda, offset=offset)
        assert np.array_equal(as_bytes(out), as_bytes(ref)), (n, offset, kind)
        assert np.array_equal(g.get_state(), end), (n, kind)


@pytest.mark.parametrize("V", [1, 2, 4])
@pytest.mark.parametrize("kind", KINDS)
def test_every_lane_layout(cuda, oracle, kind, V):
    """Every lane layout the autotuner may pick (V substreams per lane, and a
    cap on resident blocks) gives the same stream, at unaligned starts and at
    sizes around the row and tile boundaries of that layout."""
    import mrg8_gb300 as m
    from mrg8_gb300 import _lib
    lib = _lib.load()
    try:
        for bps in (0, 2):
            _lib.check(lib.mrg8g_tune_plain(kind, V, bps))
            g = m.MRG8(77 + 10 * V + kind)
            rng = np.random.default_rng(V * 10 + kind + bps)
            for n in (1, 3, 31 * V + 1, 32 * V * 8 + 5, 32 * V * 64 + 7, 1 << 20, 3_000_017):
                offset = int(rng.integers(0, 4))
                st = g.get_state()
                ref, end = oracle.generate(st, n, kind, nthreads=4)
                out = gen_device(g, n, kind, cuda, offset=offset)
                assert np.array_equal(as_bytes(out), as_bytes(ref)), (V, bps, n, offset)
                assert np.array_equal(g.get_state(), end)
    finally:
        _lib.check(lib.mrg8g_tune_plain(kind, 0, 0))


@pytest.mark.parametrize("kind", [po.U32, po.F64_SHIFTED, po.F32_ORIGINAL])
def test_consecutive_calls_continue_the_stream(cuda, oracle, kind):
    import mrg8_gb300 as m
    import torch
    g = m.MRG8(31337)
    st0 = g.get_state()
    sizes = [5, 3, 1, 8, 100, 4096, 7, 123457, 1, 2, 3, 65536 * 3 + 11]
    total = sum(sizes)
    ref, end = oracle.generate(st0, total, kind, nthreads=4)
    dt = torch_dtype(kind)
    buf = torch.empty(total, dtype=dt, device=cuda)
    off = 0
    for n in sizes:
        g._generate(buf[off:off + n], n, kind)
        off += n
    torch.cuda.synchronize()
    assert np.array_equal(as_bytes(buf), as_bytes(ref))
    assert np.array_equal(g.get_state(), end)


@pytest.mark.parametrize("m_pos", [0, 3, 7, 8, 300, 600, 1100, 5000, 100001])
def test_zero_residue_and_unit_outputs(cuda, oracle, m_pos):
    """Outputs congruent to 0 (representative p: ORIGINAL 1.0, SHIFTED
    (p-1)/p) and to 1 (SHIFTED 0.0) at positions in the head, the window rows
    and the recurrence rows."""
    import mrg8_gb300 as m
    rng = np.random.default_rng(m_pos)
    g = m.MRG8(1)
    for residue in (0, 1):
        st = state_with_output(m_pos, residue, rng)
        ints, _ = oracle.randint(st, m_pos + 1)
        assert int(ints[m_pos]) == (P if residue == 0 else 1)
        for kind in KINDS:
            for offset in (0, 1):
                g.set_state(st)
                n = m_pos + 40
                ref, end = oracle.generate(st, n, kind)
                out = gen_device(g, n, kind, cuda, offset=offset)
                assert np.array_equal(as_bytes(out), as_bytes(ref)), (residue, kind, offset)
                assert np.array_equal(g.get_state(), end)
    g.set_state(state_with_output(m_pos, 0, rng))
    import torch
    f = torch.empty(m_pos + 1, dtype=torch.float64, device=cuda)
    g.rand(f, scaling=0)
    assert float(f[m_pos]) == 1.0
    g.set_state(state_with_output(m_pos, 0, rng))
    g.rand(f, scaling=1)
    assert float(f[m_pos]) == (P - 1) / P


def test_states_with_zero_and_p_words(cuda, oracle):
    import mrg8_gb300 as m
    rng = np.random.default_rng(5)
    g = m.MRG8(1)
    for t in range(12):
        st = rng.integers(1, P, 8).astype(np.uint32)
        st[t % 8] = 0
        st[(t + 3) % 8] = P
        for n in (1, 3, 7, 9, 700, 70001):
            g.set_state(st)
            ref, end = oracle.generate(st, n, po.F64_ORIGINAL)
            out = gen_device(g, n, po.F64_ORIGINAL, cuda)
            assert np.array_equal(bits64(out.numpy()), bits64(ref)), (t, n)
            assert np.array_equal(g.get_state(), end), (t, n)


@pytest.mark.parametrize("kind", [po.F64_SHIFTED, po.F64_ORIGINAL, po.F32_SHIFTED, po.U32])
def test_full_size_2p30(cuda, oracle, kind):
    """2^30 outputs from one seed, bit-exact with the sequential
    stream (the oracle splits it over host threads by jump-ahead)."""
    import os

    import mrg8_gb300 as m
    import torch
    n = 1 << 30
    g = m.MRG8(13579)
    st = g.get_state()
    out = torch.empty(n, dtype=torch_dtype(kind), device=cuda)
    g._generate(out, n, kind)
    host = out.cpu()
    del out
    torch.cuda.empty_cache()
    ref, end = oracle.generate(st, n, kind, nthreads=os.cpu_count() or 8)
    assert np.array_equal(as_bytes(host), as_bytes(ref))
    assert np.array_equal(g.get_state(), end)


@pytest.mark.parametrize("kind", [po.F64_ORIGINAL, po.U32, po.F32_SHIFTED])
def test_host_buffer_path(cuda, oracle, kind):
    """mrg8g_generate_host: host arrays (pageable numpy and pinned torch),
    across the device staging chunks."""
    import mrg8_gb300 as m
    import torch
    g = m.MRG8(777)
    st = g.get_state()
    n = (64 << 20) // po.KIND_DTYPE[kind]().itemsize * 2 + 12345  # > two chunks
    ref, end = oracle.generate(st, n, kind, nthreads=8)
    host = np.empty(n, dtype=po.KIND_DTYPE[kind])
    g._generate(host, n, kind)
    assert np.array_equal(host.view(np.uint8), ref.view(np.uint8))
    assert np.array_equal(g.get_state(), end)
    pinned = torch.empty(1000, dtype=torch_dtype(kind)).pin_memory()
    ref2, end2 = oracle.generate(end, 1000, kind)
    g._generate(pinned, 1000, kind)
    assert np.array_equal(as_bytes(pinned), as_bytes(ref2))
    assert np.array_equal(g.get_state(), end2)
    # scalar draws of the reference API
    g.set_state(end2)
    v = g.randint()
    assert v == int(oracle.randint(end2, 1)[0][0])


def test_convert_utility(cuda, oracle):
    import mrg8_gb300 as m
    import torch
    vals = np.array([1, 2, 3, P, P - 1, 2**30, 2**30 + 1, 0x7FFFFFBF, 0x7FFFFF3F, 12345678, 2**22, 2**22 + 1],
                    dtype=np.uint32)
    vals = np.concatenate([vals, np.random.default_rng(0).integers(1, P + 1, 1 << 20).astype(np.uint32)])
    d_in = torch.from_numpy(vals.view(np.int32)).to(cuda)
    for sc in (0, 1):
        o64 = torch.empty(vals.size, dtype=torch.float64, device=cuda)
        o32 = torch.empty(vals.size, dtype=torch.float32, device=cuda)
        m.convert(d_in, o64, sc)
        m.convert(d_in, o32, sc)
        want = np.array([oracle.u31_to_f64(int(v), sc) for v in vals[:12]])
        got64 = o64.cpu().numpy()
        assert np.array_equal(bits64(got64[:12]), bits64(want))
        rnorm = 1.0 / P
        ref = (vals.astype(np.float64) - sc) * rnorm
        assert np.array_equal(bits64(got64), bits64(ref))
        assert np.array_equal(o32.cpu().numpy().view(np.uint32), ref.astype(np.float32).view(np.uint32))


def test_device_jump_states(cuda, oracle):
    """The jump prologue of 65,536 substreams: offsets drawn in [0, 2^63),
    each device state equal to the host jump A^k s."""
    import mrg8_gb300 as m
    import torch
    rng = np.random.default_rng(63)
    st = oracle.seed(13579)
    offs = rng.integers(0, 2**63, 65536, dtype=np.int64).astype(np.uint64)
    offs[:20] = np.arange(20)
    d_off = torch.from_numpy(offs.view(np.int64)).to(cuda)
    states = u32_view(m.jump_states(st, d_off))
    for i in list(range(40)) + list(rng.integers(0, 65536, 400)):
        assert states[i].tolist() == oracle.jump_matvec(st, int(offs[i])).tolist(), i
    for i in list(range(12)) + list(rng.integers(0, 65536, 8)):
        assert states[i].tolist() == oracle.jump(st, int(offs[i])).tolist(), i
