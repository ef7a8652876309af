"""Serving (continuous batching): every result equals its request's own
stream segment alone and in the mix, generator draws continue one stream,
admission respects the budget, and the load test runs."""
import threading
import time

import numpy as np
import pytest

from oracle import pyoracle as po

pytestmark = pytest.mark.gpu

KINDS = [po.U32, po.F64_ORIGINAL, po.F64_SHIFTED, po.F32_ORIGINAL, po.F32_SHIFTED]


def segment(oracle, seed, offset, n, kind):
    st = oracle.seed(seed)
    if offset >= 8:
        st = oracle.jump_matvec(st, offset)
    elif offset:
        _, st = oracle.randint(st, offset)
    out, _ = oracle.generate(st, n, kind, nthreads=4)
    return out


def drain(srv, want, results, release=True):
    while len(results) < want:
        for c in srv.poll(256, 2000):
            assert c["status"] == 0
            results[c["ticket"]] = (c, srv.read(c))
            if release:
                srv.release(c["ticket"])


def test_results_equal_alone_and_in_the_mix(cuda, oracle):
    from mrg8_gb300.serve import Server
    rng = np.random.default_rng(5)
    probes = []
    for i in range(40):
        kind = KINDS[i % 5]
        n = int(2 ** rng.uniform(0, 16))
        seed = int(rng.integers(0, 2**32))
        off = int(rng.integers(0, 2**48)) if i % 3 else int(rng.integers(0, 9))
        probes.append((seed, off, n, kind))
    # alone: one request at a time
    alone = {}
    with Server(budget_bytes=256 << 20) as srv:
        for j, (seed, off, n, kind) in enumerate(probes):
            t = srv.submit(n, kind, seed=seed, offset=off, tag=j)
            res = {}
            drain(srv, 1, res)
            alone[j] = res[t][1]
    # in the mix: the probes interleaved with a stream of background requests
    mixed = {}
    with Server(budget_bytes=256 << 20, inflight=3, max_batch=64) as srv:
        tickets = {}
        results = {}
        stop = threading.Event()

        def background():
            k = 0
            while not stop.is_set():
                srv.submit(int(2 ** rng.uniform(8, 18)), KINDS[k % 5], seed=k, offset=k * 7919)
                k += 1
                time.sleep(0.0002)

        bg = threading.Thread(target=background)
        bg.start()
        for j, (seed, off, n, kind) in enumerate(probes):
            tickets[srv.submit(n, kind, seed=seed, offset=off, tag=1000 + j)] = j
        deadline = time.time() + 60
        while len(mixed) < len(probes) and time.time() < deadline:
            for c in srv.poll(256, 2000):
                if c["tag"] >= 1000:
                    mixed[c["tag"] - 1000] = srv.read(c)
                srv.release(c["ticket"])
        stop.set()
        bg.join()
        st = srv.stats()
        assert st["launches"] >= 2 and st["error"] == 0
    for j, (seed, off, n, kind) in enumerate(probes):
        want = segment(oracle, seed, off, n, kind)
        assert np.array_equal(alone[j].view(np.uint8), want.view(np.uint8)), j
        assert np.array_equal(mixed[j].view(np.uint8), want.view(np.uint8)), j


def test_generator_draws_continue_one_stream(cuda, oracle):
    from mrg8_gb300.serve import Server
    rng = np.random.default_rng(8)
    with Server(budget_bytes=128 << 20) as srv:
        gens = [srv.add_generator(oracle.seed(100 + g)) for g in range(5)]
        draws = {g: [] for g in gens}
        tickets = {}
        for r in range(30):
            g = gens[r % 5]
            n = int(rng.integers(1, 5000))
            kind = KINDS[r % 5]
            tickets[srv.submit(n, kind, generator=g)] = (g, len(draws[g]))
            draws[g].append((n, kind))
        results = {}
        drain(srv, len(tickets), results)
        for g in gens:
            st = oracle.seed(100 + g)
            for k, (n, kind) in enumerate(draws[g]):
                want, st = oracle.generate(st, n, kind)
                tk = [t for t, v in tickets.items() if v == (g, k)][0]
                assert np.array_equal(results[tk][1].view(np.uint8), want.view(np.uint8)), (g, k)
            assert srv.generator_state(g).tolist() == st.tolist()


def test_admission_respects_the_budget(cuda, oracle):
    from mrg8_gb300 import MRG8GError
    from mrg8_gb300.serve import Server
    budget = 4 << 20
    with Server(budget_bytes=budget, inflight=2) as srv:
        with pytest.raises(MRG8GError):
            srv.submit((budget // 8) + 1, po.F64_SHIFTED, seed=1)
        n = (budget // 8) // 3  # three fit at once, not four
        ts = [srv.submit(n, po.F64_SHIFTED, seed=s, offset=s) for s in range(12)]
        results = {}
        held = []
        deadline = time.time() + 60
        while len(results) < len(ts) and time.time() < deadline:
            for c in srv.poll(16, 2000):
                results[c["ticket"]] = srv.read(c)
                held.append(c["ticket"])
            st = srv.stats()
            assert st["bytes_in_use"] <= budget
            while len(held) > 1:
                srv.release(held.pop(0))
        st = srv.stats()
        assert len(results) == len(ts), (st, sorted(results))
        for h in held:
            srv.release(h)
        assert srv.stats()["peak_bytes"] <= budget
    for s, t in enumerate(ts):
        assert np.array_equal(results[t].view(np.uint64), segment(oracle, s, s, n, po.F64_SHIFTED).view(np.uint64))


def test_space_released_behind_a_held_result_is_reused(cuda, oracle):
    """Two results fit in the arena.  The client keeps the older one and
    releases the newer; the next request must fit into the released space
    and complete (a ring arena would wait for the older one forever)."""
    from mrg8_gb300.serve import Server
    budget = 4 << 20
    n = (budget // 8) // 3
    with Server(budget_bytes=budget, inflight=2) as srv:
        first = [srv.submit(n, po.F64_SHIFTED, seed=s, offset=s) for s in range(2)]
        got = {}
        deadline = time.time() + 20
        while len(got) < 2 and time.time() < deadline:
            for c in srv.poll(4, 2000):
                got[c["ticket"]] = c
        assert sorted(got) == sorted(first)
        srv.release(first[1])           # the newer one; the older stays held
        nxt = srv.submit(n, po.F64_SHIFTED, seed=2, offset=2)
        done = []
        deadline = time.time() + 20
        while not done and time.time() < deadline:
            done = srv.poll(4, 2000)
        assert [c["ticket"] for c in done] == [nxt], srv.stats()
        out = srv.read(done[0])
        srv.release(nxt)
        srv.release(first[0])
    assert np.array_equal(out.view(np.uint64), segment(oracle, 2, 2, n, po.F64_SHIFTED).view(np.uint64))


def test_loadtest_smoke(cuda):
    from mrg8_gb300.serve import Server
    with Server(budget_bytes=2 << 30) as srv:
        r = srv.loadtest(rate=2000, duration_s=0.5, n_min=256, n_max=1 << 20, offset_max=1 << 48)
    assert r["requests"] > 500
    assert 0 < r["p50_us"] <= r["p99_us"] <= r["max_us"]
    assert r["gsamples_per_s"] > 0


def test_request_errors_are_reported(cuda):
    from mrg8_gb300 import MRG8GError
    from mrg8_gb300.serve import Server
    with Server(budget_bytes=1 << 20) as srv:
        with pytest.raises(MRG8GError):
            srv.submit(10, 9)                          # unknown kind
        with pytest.raises(MRG8GError):
            srv.submit(10, po.U32, generator=3)        # unknown generator
        with pytest.raises(MRG8GError):
            srv.submit(1 << 20, po.F64_SHIFTED)        # larger than the budget
        with pytest.raises(MRG8GError):
            srv.release(12345)                         # unknown ticket
        with pytest.raises(MRG8GError):
            srv.add_generator([0] * 8)                 # all-zero state
        t = srv.submit(1000, po.U32, seed=3)
        got = {}
        drain(srv, 1, got, release=False)
        srv.release(t)
        with pytest.raises(MRG8GError):
            srv.release(t)                             # released twice
        assert srv.stats()["error"] == 0


def test_sleeping_scheduler_gives_the_same_results(cuda, oracle):
    """spin_us < 0: the scheduler sleeps whenever nothing is in flight; requests
    spaced out in time still complete with their own stream segments."""
    from mrg8_gb300.serve import Server
    rng = np.random.default_rng(11)
    with Server(budget_bytes=64 << 20, spin_us=-1) as srv:
        for j in range(12):
            kind = KINDS[j % 5]
            n = int(2 ** rng.uniform(4, 14))
            seed = int(rng.integers(0, 2**32))
            off = int(rng.integers(0, 2**40))
            t = srv.submit(n, kind, seed=seed, offset=off, tag=j)
            res = {}
            drain(srv, 1, res)
            assert np.array_equal(res[t][1].view(np.uint8), segment(oracle, seed, off, n, kind).view(np.uint8))
            time.sleep(0.004)  # longer than any spin window: the next submit wakes a sleeping thread


def test_burst_batches_and_overlaps_on_the_device(cuda, oracle):
    """A burst of 300 mid-size requests arriving while every in-flight slot is
    busy: the scheduler packs them into few launches (mean batch > 1), keeps
    several launches in flight, their device intervals (events around each
    launch's copy and kernel) overlap, and every result still equals its
    request's own stream segment."""
    from mrg8_gb300.serve import Server
    rng = np.random.default_rng(21)
    with Server(budget_bytes=8 << 30, inflight=3, max_batch=32) as srv:
        # One large request per slot, each launched before the next is
        # submitted, so that all three slots are busy when the burst comes.
        blockers = []
        for b in range(3):
            blockers.append(srv.submit(1 << 28, po.F64_SHIFTED, seed=900 + b))
            deadline = time.time() + 10
            while srv.stats()["launches"] < b + 1 and time.time() < deadline:
                time.sleep(1e-5)
        burst = []
        for j in range(300):
            kind = KINDS[j % 5]
            n = int(2 ** rng.uniform(10, 17))
            seed = int(rng.integers(0, 2**32))
            off = int(rng.integers(0, 2**40))
            burst.append((srv.submit(n, kind, seed=seed, offset=off, tag=j), seed, off, n, kind))
        results = {}
        deadline = time.time() + 60
        while len(results) < 303 and time.time() < deadline:
            for c in srv.poll(256, 2000):
                assert c["status"] == 0
                if c["ticket"] not in blockers:
                    results[c["ticket"]] = srv.read(c)
                else:
                    results[c["ticket"]] = None
                srv.release(c["ticket"])
        st = srv.stats()
    assert len(results) == 303
    assert st["error"] == 0
    assert st["max_inflight"] >= 2, st
    assert st["mean_batch"] > 1.0, st
    assert st["overlapped_launches"] >= 2, st
    for tk, seed, off, n, kind in burst:
        want = segment(oracle, seed, off, n, kind)
        assert np.array_equal(results[tk].view(np.uint8), want.view(np.uint8)), (tk, n, kind)
