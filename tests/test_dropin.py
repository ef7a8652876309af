"""The header-only drop-in classes (include/mrg8_cuda.hpp) compiled into a
reference-style driver and linked against libmrg8g.so."""
import os
import subprocess

import numpy as np
import pytest

from conftest import ROOT
from oracle import pyoracle as po


@pytest.fixture(scope="module")
def driver(lib, tmp_path_factory):
    from mrg8_gb300 import build
    exe = str(tmp_path_factory.mktemp("dropin") / "dropin_driver")
    subprocess.run([build.nvcc(), "-std=c++17", "-O2", "-I" + os.path.join(ROOT, "include"), "-o", exe,
                    os.path.join(ROOT, "tests", "native", "dropin_driver.cpp"),
                    "-L" + build.LIBDIR, "-lmrg8g", "-Xlinker", "-rpath=" + build.LIBDIR], check=True)
    return exe


def parse(out):
    rows = {}
    for line in out.splitlines():
        parts = line.split()
        rows[parts[0]] = parts[1:]
    return rows


def test_dropin_host_calls(driver, oracle):
    r = subprocess.run([driver, "host"], capture_output=True, text=True, check=True)
    rows = parse(r.stdout)
    st = oracle.seed(13579)
    assert [int(v) for v in rows["seeded"]] == st.tolist()
    j = oracle.jump(st, 1000)
    assert [int(v) for v in rows["jump1000"]] == j.tolist()
    assert [int(v) for v in rows["after_jump"]] == j.tolist()
    assert [int(v) for v in rows["after_jump2^199"]] == oracle.jump_bits(j, [0] * 199 + [1]).tolist()


def digest(a: np.ndarray) -> int:
    """sum_i word_i * (2 i + 1) mod 2^64 over the 8-byte words of a (as the driver)."""
    w = a.view(np.uint64)
    with np.errstate(over="ignore"):
        return int((w * (2 * np.arange(w.size, dtype=np.uint64) + np.uint64(1))).sum(dtype=np.uint64))


@pytest.mark.gpu
def test_dropin_mrg8dnz2_both_scalings(driver, oracle):
    """mrg8::mrg8dnz2 of the compiled drop-in against the oracle's restatement
    of cuda/mrg8.cpp:290-339 (ORIGINAL) and knl/mrg8.h:387-436 (SHIFTED), on
    consecutive calls of sizes around the reference's 1024-deep buffer."""
    r = subprocess.run([driver, "dnz2"], capture_output=True, text=True, check=True)
    rows = parse(r.stdout)
    for scaling in (0, 1):
        st = oracle.seed(13579)
        for n in (1, 1023, 1024, 1025, 3000, 1000000):
            want, st = oracle.mrg8dnz2(st, n, scaling)
            got = rows[f"dnz2_{scaling}_{n}"]
            assert float(got[1]) == want[-1], (scaling, n)
            assert int(got[0]) == digest(want), (scaling, n)
        assert [int(v) for v in rows[f"dnz2_state_{scaling}"]] == st.tolist()


@pytest.mark.gpu
def test_dropin_device_and_host_generation(driver, oracle):
    r = subprocess.run([driver, "gpu"], capture_output=True, text=True, check=True)
    rows = parse(r.stdout)
    st = oracle.seed(13579)
    n = 1 << 20
    sh, end = oracle.generate(st, n, po.F64_SHIFTED)
    assert [int(v) for v in rows["after_outer"]] == end.tolist()
    assert float(rows["outer_first"][0]) == sh[0] and float(rows["outer_first"][1]) == sh[1]
    assert float(rows["outer_first"][3]) == sh[-1]
    assert rows["inner_equals_outer"] == ["1"]
    f, e1 = oracle.rand_f64(st, 1000, 0)
    assert float(rows["rand_first"][0]) == f[0] and float(rows["rand_first"][2]) == f[999]
    ints, e2 = oracle.randint(e1, 10)
    assert [int(v) for v in rows["randint"]] == ints.tolist()
    a, e3 = oracle.randint(e2, 1)
    b, e4 = oracle.rand_f64(e3, 2, 0)
    assert int(rows["scalar"][0]) == int(a[0])
    assert float(rows["scalar"][1]) == b[0] and float(rows["scalar"][2]) == b[1]
    assert [int(v) for v in rows["final"]] == e4.tolist()
