"""The C-ABI library: loads, exports every declared symbol, and its host-side
logic (seeding, state, jumps, argument checks) matches the oracle.  None of
these calls touches a GPU."""
import ctypes as C
import os
import re

import numpy as np
import pytest

from conftest import ROOT

P = 2147483647


def declared_symbols():
    names = set()
    for f in os.listdir(os.path.join(ROOT, "include")):
        if f.endswith(".h"):
            text = open(os.path.join(ROOT, "include", f)).read()
            names |= set(re.findall(r"MRG8G_API\s+[\w\s\*]+?\b(mrg8g_\w+)\s*\(", text))
    return names


def test_exports_every_declared_symbol(lib):
    names = declared_symbols()
    assert len(names) >= 18
    from mrg8_gb300._lib import SIGNATURES
    for n in names:
        assert hasattr(lib, n), n
        assert n in SIGNATURES, f"{n} has no ctypes signature"
    assert lib.mrg8g_version() == 1


def test_ctypes_structs_match_the_header(tmp_path):
    """Every ctypes mirror in mrg8_gb300/_lib.py has the size and the field
    offsets that a C compiler gives the struct of include/mrg8g.h."""
    import subprocess

    from mrg8_gb300 import _lib as L
    mirrors = {}
    for name in dir(L):
        cls = getattr(L, name)
        if isinstance(cls, type) and issubclass(cls, C.Structure) and cls.__doc__:
            m = re.match(r"(mrg8g_\w+) of include/mrg8g\.h", cls.__doc__)
            if m:
                mirrors[m.group(1)] = cls
    assert len(mirrors) >= 8, sorted(mirrors)
    lines = ["#include <stddef.h>", "#include <stdio.h>", '#include "mrg8g.h"', "int main(void) {"]
    for cname, cls in sorted(mirrors.items()):
        lines.append(f'printf("{cname} size %zu\\n", sizeof({cname}));')
        for f, _ in cls._fields_:
            lines.append(f'printf("{cname} {f} %zu\\n", offsetof({cname}, {f}));')
    lines.append("return 0; }")
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines))
    exe = tmp_path / "layout"
    subprocess.run(["gcc", "-std=c11", "-I" + os.path.join(ROOT, "include"), "-o", str(exe), str(src)], check=True)
    got = {}
    for line in subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.splitlines():
        cname, field, value = line.split()
        got[(cname, field)] = int(value)
    for cname, cls in mirrors.items():
        assert got[(cname, "size")] == C.sizeof(cls), cname
        for f, _ in cls._fields_:
            assert got[(cname, f)] == getattr(cls, f).offset, (cname, f)


def test_seeding_and_state(lib, oracle, kat):
    import mrg8_gb300 as m
    for seed, st in kat["seed_states"].items():
        g = m.MRG8(int(seed))
        assert g.get_state().tolist() == st
        g.seed_init(13579)
        assert g.get_state().tolist() == kat["seed_states"]["13579"]
    g = m.MRG8Cuda(13579)
    buf = np.zeros(8, dtype=np.uint32)
    g.get_state(buf)
    assert buf.tolist() == kat["seed_states"]["13579"]
    st = [5, 0, 7, P, 9, 10, 11, 12]
    g.set_state(st)
    assert g.get_state().tolist() == st


@pytest.mark.parametrize("bad", [[0] * 8, [2**31] + [1] * 7, [1] * 7 + [2**32 - 1]])
def test_invalid_states_rejected(lib, bad):
    import mrg8_gb300 as m
    g = m.MRG8(1)
    before = g.get_state()
    with pytest.raises(m.MRG8GError) as e:
        g.set_state(bad)
    assert e.value.code == -2
    assert np.array_equal(g.get_state(), before)


def test_jumps_known_answers(lib, kat):
    import mrg8_gb300 as m
    g = m.MRG8(1)
    for j in kat["jumps"]:
        k = int(j["k"])
        g.set_state(j["state"])
        out = np.zeros(8, dtype=np.uint32)
        g.jump_ahead(k, out)                         # cuda/knl out-parameter form
        assert out.tolist() == j["original"]
        assert g.get_state().tolist() == j["state"]
        g.jump_ahead(k)                              # original/ mutating form
        assert g.get_state().tolist() == j["original"]
    for j in kat["jumps200"]:
        g.set_state(j["state"])
        b = [int(c) for c in j["bits"]]
        out = np.zeros(8, dtype=np.uint32)
        g.jump_ahead(b, out)
        assert out.tolist() == j["original"]
        k = sum(bit << i for i, bit in enumerate(b))
        g.jump_ahead(k)
        assert g.get_state().tolist() == j["original"]


def test_jumps_random_against_oracle(lib, oracle):
    import mrg8_gb300 as m
    rng = np.random.default_rng(11)
    g = m.MRG8(3)
    for t in range(200):
        st = rng.integers(0, 2**31, 8, dtype=np.int64).astype(np.uint32)
        if t % 4 == 0:
            st[t % 8] = 0
        if t % 9 == 0:
            st[(t + 1) % 8] = P
        if not st.any():
            st[0] = 1
        k = int(rng.integers(0, 2**63)) if t % 2 else int(rng.integers(0, 20))
        g.set_state(st)
        g.jump_ahead(k)
        assert np.array_equal(g.get_state(), oracle.jump(st, k)), (t, k)


def test_argument_errors(lib):
    import mrg8_gb300 as m
    from mrg8_gb300 import _lib as L
    assert lib.mrg8g_seed_init(None, 1) == L.ERR_INVALID_ARGUMENT
    assert b"null generator" in lib.mrg8g_last_error()
    g = m.MRG8(1)
    assert lib.mrg8g_generate(g.handle, C.c_void_p(0), 10, 9, None) == L.ERR_INVALID_ARGUMENT
    assert lib.mrg8g_rand(g.handle, C.c_void_p(0), 10, 7, None) == L.ERR_INVALID_ARGUMENT
    assert lib.mrg8g_convert(C.c_void_p(0), C.c_void_p(0), 10, 0, None) == L.ERR_INVALID_ARGUMENT
    assert lib.mrg8g_generate(g.handle, C.c_void_p(0), 0, 1, None) == L.SUCCESS  # n = 0 is a no-op
    assert lib.mrg8g_generate(g.handle, C.c_void_p(0), (1 << 62) + 1, 1, None) == L.ERR_INVALID_ARGUMENT
    with pytest.raises(ValueError):
        m.MRG8Cuda(1).mrg8_outer_32(np.zeros(4), 4, 48, 1024)
    with pytest.raises(ValueError):
        g.jump_ahead(1 << 200)


def test_missing_library_fails_loudly(tmp_path, monkeypatch):
    from mrg8_gb300 import _lib as L
    monkeypatch.setattr(L, "LIB_PATH", str(tmp_path / "absent.so"))
    monkeypatch.setattr(L, "_lib", None)
    with pytest.raises(OSError, match="no CPU fallback"):
        L.load()


def test_jump_matrix_file_round_trip(lib, oracle, tmp_path, kat):
    """The reference's jump_matrix.txt format: the written table parses to the
    oracle's table (which the golden digest pins to the reference's file), a
    corrupted entry is reported, and the reference's own file verifies where
    it is present."""
    import hashlib
    from mrg8_gb300 import _lib as L
    from oracle.pyoracle import reference_dir
    path = tmp_path / "jump_matrix.txt"
    assert lib.mrg8g_write_jump_matrix(str(path).encode()) == 0
    tab = oracle.read_jump_matrix(str(path))
    assert np.array_equal(tab, oracle.tab)
    assert hashlib.sha256(tab.astype(np.uint32).tobytes()).hexdigest() == kat["jump_matrix_txt"]["sha256_u32"]
    bad = C.c_uint64()
    assert lib.mrg8g_verify_jump_matrix(str(path).encode(), C.byref(bad)) == 0 and bad.value == 0
    vals = path.read_text().split()
    vals[1000] = str(int(vals[1000]) + 1)
    path.write_text(" ".join(vals))
    assert lib.mrg8g_verify_jump_matrix(str(path).encode(), C.byref(bad)) == L.ERR_INVALID_STATE
    assert bad.value == 1
    refdir = reference_dir()
    ref = os.path.join(refdir, "original", "jump_matrix.txt") if refdir else None
    if ref and os.path.exists(ref):
        assert lib.mrg8g_verify_jump_matrix(ref.encode(), C.byref(bad)) == 0
