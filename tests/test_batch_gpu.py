"""The batch path (one persistent, graph-captured launch for many independent
instances) against the oracle and against the per-instance bulk path."""
import numpy as np
import pytest

from mrg8_helpers import P
from oracle import pyoracle as po

pytestmark = pytest.mark.gpu

KINDS = [po.U32, po.F64_ORIGINAL, po.F64_SHIFTED, po.F32_ORIGINAL, po.F32_SHIFTED]
ELEM = {po.U32: 4, po.F64_ORIGINAL: 8, po.F64_SHIFTED: 8, po.F32_ORIGINAL: 4, po.F32_SHIFTED: 4}


def tdt(kind):
    import torch
    if kind == po.U32:
        return torch.int32
    return torch.float64 if ELEM[kind] == 8 else torch.float32


def as_bytes(t):
    return t.detach().cpu().numpy().view(np.uint8)


def expected(oracle, state, offset, n, kind):
    st = oracle.jump_matvec(state, offset) if offset else np.asarray(state, dtype=np.uint32)
    if offset and offset < 8:
        st = np.asarray(state, dtype=np.uint32)
        _, st = oracle.randint(st, offset)
    out, _ = oracle.generate(st, n, kind, nthreads=4)
    return out


def make_instances(cuda, rng, count, max_log2, offsets=True):
    import torch
    import mrg8_gb300 as m
    insts, meta = [], []
    for i in range(count):
        kind = KINDS[int(rng.integers(0, 5))]
        n = int(2 ** rng.uniform(0, max_log2)) if i % 7 else int(rng.choice([0, 1, 2, 3, 5, 7, 8, 9, 31, 129]))
        off = 0
        if offsets and i % 3 == 0:
            off = int(rng.integers(0, 2**63)) if i % 2 else int(rng.integers(0, 10))
        lead = int(rng.integers(0, 4))
        buf = torch.full((n + lead + 3,), -5, dtype=tdt(kind), device=cuda)
        seed = int(rng.integers(0, 2**32))
        st = m.seed_state(seed)
        insts.append((st, off, buf[lead:lead + n], kind))
        meta.append((st, off, n, kind, buf, lead))
    return insts, meta


def check_canaries(meta):
    import torch
    for st, off, n, kind, buf, lead in meta:
        host = buf.cpu()
        fill = torch.full((1,), -5, dtype=buf.dtype)
        assert bool((host[:lead] == fill).all()) and bool((host[lead + n:] == fill).all())


def test_batch_matches_oracle(cuda, oracle):
    import torch
    import mrg8_gb300 as m
    rng = np.random.default_rng(4)
    insts, meta = make_instances(cuda, rng, 160, 17)
    b = m.Batch(insts)
    b.launch()
    torch.cuda.synchronize()
    for (st, off, n, kind, buf, lead), (_, _, view, _) in zip(meta, insts):
        want = expected(oracle, st, off, n, kind)
        assert np.array_equal(as_bytes(view), want.view(np.uint8)), (off, n, kind, lead)
    check_canaries(meta)
    st = b.stats()
    assert st["outputs"] == sum(x[2] for x in meta)


def test_replan_right_after_a_launch_on_a_non_blocking_stream(cuda, oracle):
    """Outputs cleared and a launch enqueued on a side stream, then at once a
    re-plan (new tile rows and tiling) from the host: the re-plan waits for
    the launch before it rewrites the descriptors, so the launch still writes
    every output of the old plan; repeated over four plans."""
    import torch

    import mrg8_gb300 as m
    rng = np.random.default_rng(31)
    insts, meta = make_instances(cuda, rng, 60, 20)
    want = [expected(oracle, st, off, n, kind).view(np.uint8) for st, off, n, kind, _, _ in meta]
    b = m.Batch(insts, tile_rows=64)
    side = torch.cuda.Stream()
    plans = ((64, 0), (16, 1), (512, 0), (32, 1), (64, 0))
    for k in range(len(plans) - 1):
        torch.cuda.synchronize()
        with torch.cuda.stream(side):
            for _, _, n, _, buf, lead in meta:
                buf[lead:lead + n].zero_()
        b.launch(stream=side)
        b.set_config(tile_rows=plans[k + 1][0], tiling=plans[k + 1][1])
        torch.cuda.synchronize()
        for (st, off, n, kind, buf, lead), w in zip(meta, want):
            assert np.array_equal(as_bytes(buf[lead:lead + n]), w), (k, n, kind, off)
    check_canaries(meta)
    b.close()


def test_batch_relaunch_autotune_and_plain_launch_agree(cuda, oracle):
    import torch
    import mrg8_gb300 as m
    rng = np.random.default_rng(9)
    insts, meta = make_instances(cuda, rng, 60, 19)
    b = m.Batch(insts)
    b.launch()
    torch.cuda.synchronize()
    first = [as_bytes(v).copy() for (_, _, v, _) in insts]
    for (_, _, v, _) in insts:
        v.zero_()
    b.launch()
    b.launch()
    torch.cuda.synchronize()
    assert all(np.array_equal(as_bytes(v), f) for (_, _, v, _), f in zip(insts, first))
    cfg = b.autotune()
    assert cfg["tile_rows"] in (128, 256, 512, 1024, 2048)
    for (_, _, v, _) in insts:
        v.zero_()
    b.launch()
    torch.cuda.synchronize()
    assert all(np.array_equal(as_bytes(v), f) for (_, _, v, _), f in zip(insts, first))
    nog = m.Batch(insts, tile_rows=64, threads=256, use_graph=False)
    for (_, _, v, _) in insts:
        v.zero_()
    nog.launch()
    torch.cuda.synchronize()
    assert all(np.array_equal(as_bytes(v), f) for (_, _, v, _), f in zip(insts, first))
    # the per-instance bulk path gives the same values
    for (st, off, v, kind), f in zip(insts, first):
        v.zero_()
        m.generate_from_state(st, off, v, kind)
    torch.cuda.synchronize()
    assert all(np.array_equal(as_bytes(v), f) for (_, _, v, _), f in zip(insts, first))
    check_canaries(meta)


@pytest.mark.parametrize("tile_rows,threads", [(16, 128), (24, 256), (512, 128)])
def test_device_derived_tiles_match_oracle(cuda, oracle, tile_rows, threads):
    """Tiles derived by the kernel from per-instance tile counts (unaligned
    heads, zero and tiny lengths, random offsets, more than 32 instances so
    that the owner search takes two levels) give every instance its own
    sequential stream, and switching a plan between the two tilings keeps
    the values."""
    import torch
    import mrg8_gb300 as m
    rng = np.random.default_rng(77 + tile_rows)
    insts, meta = make_instances(cuda, rng, 90, 16)
    b = m.Batch(insts, tile_rows=tile_rows, threads=threads, tiling=1)
    assert b.config["tiling"] == 1
    b.launch()
    torch.cuda.synchronize()
    for (st, off, n, kind, buf, lead), (_, _, view, _) in zip(meta, insts):
        want = expected(oracle, st, off, n, kind)
        assert np.array_equal(as_bytes(view), want.view(np.uint8)), (off, n, kind, lead)
    check_canaries(meta)
    first = [as_bytes(v).copy() for (_, _, v, _) in insts]
    for tiling in (0, 1):
        assert b.set_config(tiling=tiling)["tiling"] == tiling
        for (_, _, v, _) in insts:
            v.zero_()
        b.launch()
        torch.cuda.synchronize()
        assert all(np.array_equal(as_bytes(v), f) for (_, _, v, _), f in zip(insts, first)), tiling
    check_canaries(meta)


def test_uneven_batch_distribution_small(cuda, oracle):
    """The uneven-batch distribution at reduced scale: distinct seeds, lengths
    log-uniform in [1, 2^18], dtypes mixed uniformly; every instance equal to
    its own sequential stream."""
    import torch
    import mrg8_gb300 as m
    rng = np.random.default_rng(2024)
    insts = []
    for i in range(1500):
        kind = [po.F64_SHIFTED, po.F32_SHIFTED, po.U32][int(rng.integers(0, 3))]
        n = max(1, int(2 ** rng.uniform(0, 18)))
        out = torch.empty(n, dtype=tdt(kind), device=cuda)
        insts.append((m.seed_state(i * 2654435761 % 2**32), 0, out, kind))
    b = m.Batch(insts)
    b.autotune()
    for (_, _, v, _) in insts:
        v.fill_(0)
    b.launch()
    torch.cuda.synchronize()
    for j in list(range(0, 1500, 37)) + [1499]:
        st, _, v, kind = insts[j]
        want, _ = oracle.generate(st, v.numel(), kind, nthreads=4)
        assert np.array_equal(as_bytes(v), want.view(np.uint8)), j


def test_batch_edge_cases_and_errors(cuda):
    import torch
    import mrg8_gb300 as m
    empty = m.Batch([])
    empty.launch()
    z = torch.empty(0, dtype=torch.float64, device=cuda)
    m.Batch([(m.seed_state(1), 0, z, po.F64_SHIFTED)]).launch()
    buf = torch.empty(16, dtype=torch.float64, device=cuda)
    with pytest.raises(ValueError):
        m.Batch([(m.seed_state(1), 0, buf, 9)])
    with pytest.raises(m.MRG8GError):
        m.Batch([([0] * 8, 0, buf, po.F64_SHIFTED)])
    with pytest.raises(m.MRG8GError):
        m.Batch([(m.seed_state(1), 2**64 - 5, buf, po.F64_SHIFTED)])
    torch.cuda.synchronize()


def test_jump_stress_65536_substreams(cuda, oracle):
    """65,536 substreams of one seed, each jumped by an offset drawn
    uniformly in [0, 2^63), 4,096 uint32 outputs each (2^28 outputs, 1 GiB).
    Every device post-jump state equals the host jump A^k s, the first eight
    outputs of every substream continue from that state, and whole substreams
    of a random subset equal the oracle."""
    import torch

    import mrg8_gb300 as m
    rng = np.random.default_rng(20240331)
    count, n = 65536, 4096
    st = oracle.seed(13579)
    offs = rng.integers(0, 2**63, count, dtype=np.int64).astype(np.uint64)
    out = torch.empty((count, n), dtype=torch.int32, device=cuda)
    b = m.Batch([(st, int(offs[i]), out[i], po.U32) for i in range(count)])
    b.launch()
    d_off = torch.from_numpy(offs.view(np.int64)).to(cuda)
    states = m.jump_states(st, d_off).cpu().numpy().view(np.uint32)
    torch.cuda.synchronize()
    host = out.cpu().numpy().view(np.uint32)
    for i in range(count):
        js = oracle.jump_matvec(st, int(offs[i]))
        assert states[i].tolist() == js.tolist(), i
        first, _ = oracle.randint(js, 8)
        assert host[i, :8].tolist() == first.tolist(), i
    for i in rng.integers(0, count, 300):
        want, _ = oracle.randint(oracle.jump_matvec(st, int(offs[i])), n)
        assert np.array_equal(host[i], want), i
    b.close()


def test_plan_limits_and_refused_configs_keep_the_plan(cuda):
    """An instance of 2^45 outputs needs 2^30 body tiles: a host-listed plan is
    refused before anything is built, the derived tiling plans it with
    O(instances) descriptors, and a refused re-plan leaves that plan and its
    configuration in place.  Through the C ABI (the Python mirror already
    refuses an n beyond its tensor); never launched, the output buffer being a
    stand-in."""
    import ctypes as C

    import torch

    import mrg8_gb300 as m
    from mrg8_gb300 import _lib as L
    lib = m.load()
    buf = torch.empty(1024, dtype=torch.int32, device=cuda)
    inst = L.Instance()
    inst.state[:] = [int(v) for v in m.seed_state(3)]
    inst.offset, inst.n, inst.out, inst.kind, inst.reserved = 0, 1 << 45, buf.data_ptr(), L.U32, 0
    arr = (L.Instance * 1)(inst)
    h = C.c_void_p()
    listed = L.BatchConfig(512, 128, 0, 1, 0)
    assert lib.mrg8g_batch_create(arr, 1, C.byref(listed), C.byref(h)) == L.ERR_INVALID_ARGUMENT
    assert b"tiling = 1" in lib.mrg8g_last_error()
    derived = L.BatchConfig(512, 128, 0, 1, 1)
    assert lib.mrg8g_batch_create(arr, 1, C.byref(derived), C.byref(h)) == 0, lib.mrg8g_last_error()
    tiles = C.c_uint64()
    assert lib.mrg8g_batch_stats(h, C.byref(tiles), None, None) == 0
    assert tiles.value == (1 << 45) // (512 * 64)
    assert lib.mrg8g_batch_set_config(h, C.byref(listed)) == L.ERR_INVALID_ARGUMENT
    got = L.BatchConfig()
    assert lib.mrg8g_batch_get_config(h, C.byref(got)) == 0
    assert (got.tile_rows, got.tiling) == (512, 1)
    assert lib.mrg8g_batch_destroy(h) == 0
