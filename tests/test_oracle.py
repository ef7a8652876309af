"""The CPU oracle pinned against the reference's golden vectors and the
reference itself (kenmiura/mrg8 compiled from its own sources)."""
import hashlib

import numpy as np
import pytest

from oracle import pyoracle as po

P = 2147483647


def sha(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def bits(a):
    return [f"{int(v):016x}" for v in np.asarray(a, dtype=np.float64).view(np.uint64)]


def test_seed_states(oracle, kat):
    for seed, st in kat["seed_states"].items():
        assert oracle.seed(int(seed)).tolist() == st, seed


def test_stream_known_answers(oracle, kat):
    k = kat["seed13579"]
    st = oracle.seed(13579)
    n = 1 << 24
    ints, end = oracle.generate(st, n, po.U32, nthreads=4)
    assert ints[:64].tolist() == k["randint_first64"]
    for i, v in k["randint_at"].items():
        assert int(ints[int(i)]) == v
    assert end.tolist() == k["state_after_2^24"]
    assert int(ints.min()) == k["min_2^24"] and int(ints.max()) == k["max_2^24"]
    assert int(ints.astype(np.uint64).sum()) == k["sum_2^24"]
    assert sha(ints) == k["sha256_randint_2^24"]


def test_uniform_known_answers(oracle, kat):
    k = kat["seed13579"]
    st = oracle.seed(13579)
    n = 1 << 24
    fo, _ = oracle.generate(st, n, po.F64_ORIGINAL, nthreads=4)
    fs, _ = oracle.generate(st, n, po.F64_SHIFTED, nthreads=4)
    assert bits(fo[:16]) == k["rand_original_first16_bits"]
    assert bits(fo[-1:])[0] == k["rand_original_at_2^24-1_bits"]
    assert sha(fo) == k["sha256_rand_original_2^24"]
    assert bits(fs[:16]) == k["rand_shifted_first16_bits"]
    assert sha(fs) == k["sha256_rand_shifted_2^24"]
    f32o, _ = oracle.generate(st, n, po.F32_ORIGINAL, nthreads=4)
    f32s, _ = oracle.generate(st, n, po.F32_SHIFTED, nthreads=4)
    assert sha(f32o) == k["sha256_f32_original_2^24"]
    assert sha(f32s) == k["sha256_f32_shifted_2^24"]


def test_sequential_entry_points_match(oracle, kat):
    st = oracle.seed(13579)
    a, e1 = oracle.randint(st, 5000)
    b, e2 = oracle.generate(st, 5000, po.U32, nthreads=1)
    assert np.array_equal(a, b) and np.array_equal(e1, e2)
    f, _ = oracle.rand_f64(st, 16, 0)
    assert bits(f) == kat["seed13579"]["rand_original_first16_bits"]
    v, end = oracle.randint(st, 1)
    assert int(v[0]) == kat["seed13579"]["randint_scalar"]["value"]
    assert end.tolist() == kat["seed13579"]["randint_scalar"]["state"]


def test_jumps_known_answers(oracle, kat):
    for j in kat["jumps"]:
        k = int(j["k"])
        assert oracle.jump(j["state"], k).tolist() == j["original"], (j["from"], k)
        assert oracle.jump_matvec(j["state"], k).tolist() == j["knl"], (j["from"], k)
    for j in kat["jumps200"]:
        b = [int(c) for c in j["bits"]]
        assert oracle.jump_bits(j["state"], b).tolist() == j["original"]
        assert j["cudahost"] == j["original"]
    after, _ = oracle.randint(oracle.jump(oracle.seed(13579), 5), 8)
    assert after.tolist() == kat["jump5_then_randint8"]
    ints, _ = oracle.randint(oracle.seed(13579), 13)
    assert ints[5:13].tolist() == kat["jump5_then_randint8"]


def test_mrg8dnz2_known_answers(oracle, kat):
    k = kat["mrg8dnz2_3000"]
    st = oracle.seed(13579)
    d, e = oracle.mrg8dnz2(st, 3000, 0)
    assert sha(d) == k["original_sha256"] and e.tolist() == k["original_state"]
    assert bits(d[-4:]) == k["original_last4_bits"]
    d, e = oracle.mrg8dnz2(st, 3000, 1)
    assert sha(d) == k["shifted_sha256"] and e.tolist() == k["shifted_state"]
    assert bits(d[:4]) == k["shifted_first4_bits"]


def test_generated_table_equals_reference_file(oracle, kat):
    t = kat["jump_matrix_txt"]
    tab = oracle.tab
    assert tab.size == t["count"]
    assert int(tab.astype(np.uint64).sum()) == t["sum"]
    assert sha(tab.astype(np.uint32)) == t["sha256_u32"]
    assert tab[:16].tolist() == t["entries_0_16"]
    assert tab[246 * 64: 246 * 64 + 8].tolist() == t["matrix246_first8"]


@pytest.mark.parametrize("kind", range(5))
@pytest.mark.parametrize("nthreads", [1, 2, 3, 7])
def test_block_split_equals_sequential(oracle, kind, nthreads):
    st = oracle.seed(424242)
    for n in (0, 1, 7, 8, 9, 63, 64, 65, 1000, 100003):
        a, ea = oracle.generate(st, n, kind, nthreads=1)
        b, eb = oracle.generate(st, n, kind, nthreads=nthreads)
        assert np.array_equal(a.view(np.uint8), b.view(np.uint8)), (n, kind, nthreads)
        assert np.array_equal(ea, eb)
    ref, _ = oracle.randint(st, 100003)
    g, _ = oracle.generate(st, 100003, po.U32, nthreads=nthreads)
    assert np.array_equal(ref, g)


def test_against_reference_build(oracle, reflib):
    ro, rc, rk = reflib["original"], reflib["cudahost"], reflib["knl"]
    rng = np.random.default_rng(7)
    for t in range(60):
        st = rng.integers(0, 2**31, 8, dtype=np.int64).astype(np.uint32)
        if t % 5 == 0:
            st[t % 8] = 0
        if t % 6 == 0:
            st[(t + 3) % 8] = P
        if not st.any():
            st[0] = 1
        n = int(rng.integers(1, 3000))
        a, ea = oracle.randint(st, n)
        b, eb = ro.randint(st, n)
        assert np.array_equal(a, b) and np.array_equal(ea, eb)
        f, _ = oracle.rand_f64(st, n, 0)
        g, _ = ro.rand(st, n)
        assert np.array_equal(f.view(np.uint64), g.view(np.uint64))
        f, _ = oracle.rand_f64(st, n, 1)
        g, _ = rk.rand(st, n)
        assert np.array_equal(f.view(np.uint64), g.view(np.uint64))
        k = int(rng.integers(0, 2**64, dtype=np.uint64)) if t % 2 else int(rng.integers(0, 40))
        assert np.array_equal(oracle.jump(st, k), ro.jump(st, k))
        assert np.array_equal(oracle.jump_matvec(st, k), rk.jump(st, k))
        d, ed = oracle.mrg8dnz2(st, n + 1024, 0)
        d2, ed2 = rc.mrg8dnz2(st, n + 1024)
        assert np.array_equal(d, d2) and np.array_equal(ed, ed2)
    st = oracle.seed(99)
    x, e = oracle.generate(st, 1 << 20, po.F64_SHIFTED, nthreads=4)
    y, e2 = rk.rand_tp(st, 1 << 20, 4)
    assert np.array_equal(x.view(np.uint64), y.view(np.uint64)) and np.array_equal(e, e2)
