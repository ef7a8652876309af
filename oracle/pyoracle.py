"""ctypes wrappers around the CPU oracle (test infrastructure only).

``Oracle`` loads ``oracle/_build/libmrg8_oracle.so`` (the C restatement in
``mrg8_oracle.c``, built with ``make -C oracle``).  ``RefLib`` loads one of the
reference builds in ``oracle/_ref/`` (kenmiura/mrg8 compiled from its own
sources by ``make -C oracle ref``); those only exist where the reference
sources were present at build time.

Only tests/, ``__graft_entry__.smoke()`` and bench.py's CPU legs import this
module, as the oracle for comparisons or as the timed CPU baseline.  The
product never does.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libmrg8_oracle.so")
REF_DIR = os.path.join(HERE, "_ref")

P = 2147483647
U32, F64_ORIGINAL, F64_SHIFTED, F32_ORIGINAL, F32_SHIFTED = range(5)
KIND_DTYPE = {
    U32: np.uint32,
    F64_ORIGINAL: np.float64,
    F64_SHIFTED: np.float64,
    F32_ORIGINAL: np.float32,
    F32_SHIFTED: np.float32,
}

_u32p = C.POINTER(C.c_uint32)


def _ptr(a: np.ndarray):
    return a.ctypes.data_as(C.c_void_p)


def _st(state) -> np.ndarray:
    a = np.ascontiguousarray(np.asarray(state, dtype=np.uint32))
    assert a.shape == (8,)
    return a.copy()


def build_oracle() -> str:
    """Compile the C restatement (idempotent)."""
    subprocess.run(["make", "-s", "-C", HERE, "all"], check=True)
    return LIB_PATH


class Oracle:
    """The C restatement of the reference algorithm."""

    _lib = None

    def __init__(self):
        if Oracle._lib is None:
            if not os.path.exists(LIB_PATH):
                build_oracle()
            lib = C.CDLL(LIB_PATH)
            lib.orc_seed.argtypes = [C.c_uint32, C.c_void_p]
            lib.orc_dot.argtypes = [C.c_void_p, C.c_void_p]
            lib.orc_dot.restype = C.c_uint32
            lib.orc_randint.argtypes = [C.c_void_p, C.c_void_p, C.c_uint64]
            lib.orc_rand_f64.argtypes = [C.c_void_p, C.c_void_p, C.c_uint64, C.c_int]
            lib.orc_rand_f32.argtypes = [C.c_void_p, C.c_void_p, C.c_uint64, C.c_int]
            lib.orc_u31_to_f64.argtypes = [C.c_uint32, C.c_int]
            lib.orc_u31_to_f64.restype = C.c_double
            lib.orc_mrg8dnz2.argtypes = [C.c_void_p, C.c_void_p, C.c_uint64, C.c_int]
            lib.orc_jump_table.argtypes = [C.c_void_p]
            lib.orc_read_jump_matrix.argtypes = [C.c_char_p, C.c_void_p]
            lib.orc_read_jump_matrix.restype = C.c_int
            lib.orc_jump_calc.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p]
            lib.orc_jump_ahead_bits.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p]
            lib.orc_jump_ahead.argtypes = [C.c_void_p, C.c_void_p, C.c_uint64]
            lib.orc_jump_ahead_matvec.argtypes = [C.c_void_p, C.c_void_p, C.c_uint64, C.c_void_p]
            lib.orc_generate.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_uint64, C.c_int, C.c_int]
            Oracle._lib = lib
        self.lib = Oracle._lib
        self.tab = np.zeros(247 * 64, dtype=np.uint32)
        self.lib.orc_jump_table(_ptr(self.tab))

    # -- seeding and state ------------------------------------------------
    def seed(self, seed: int) -> np.ndarray:
        st = np.zeros(8, dtype=np.uint32)
        self.lib.orc_seed(C.c_uint32(seed & 0xFFFFFFFF), _ptr(st))
        return st

    def dot(self, x, y) -> int:
        return int(self.lib.orc_dot(_ptr(_st(x)), _ptr(_st(y))))

    # -- sequential generation (state in, outputs and end state out) -------
    def randint(self, state, n: int):
        st = _st(state)
        out = np.empty(n, dtype=np.uint32)
        self.lib.orc_randint(_ptr(st), _ptr(out), C.c_uint64(n))
        return out, st

    def rand_f64(self, state, n: int, scaling: int):
        st = _st(state)
        out = np.empty(n, dtype=np.float64)
        self.lib.orc_rand_f64(_ptr(st), _ptr(out), C.c_uint64(n), scaling)
        return out, st

    def rand_f32(self, state, n: int, scaling: int):
        st = _st(state)
        out = np.empty(n, dtype=np.float32)
        self.lib.orc_rand_f32(_ptr(st), _ptr(out), C.c_uint64(n), scaling)
        return out, st

    def mrg8dnz2(self, state, n: int, scaling: int):
        st = _st(state)
        out = np.empty(n, dtype=np.float64)
        self.lib.orc_mrg8dnz2(_ptr(st), _ptr(out), C.c_uint64(n), scaling)
        return out, st

    def u31_to_f64(self, s: int, scaling: int) -> float:
        return float(self.lib.orc_u31_to_f64(C.c_uint32(s), scaling))

    # -- block-split generation (same stream, many threads) -----------------
    def generate(self, state, n: int, kind: int, nthreads: int = 1, out=None):
        st = _st(state)
        if out is None:
            out = np.empty(n, dtype=KIND_DTYPE[kind])
        assert out.dtype == KIND_DTYPE[kind] and out.size >= n and out.flags.c_contiguous
        self.lib.orc_generate(_ptr(st), _ptr(self.tab), _ptr(out), C.c_uint64(n), kind, nthreads)
        return out, st

    # -- jumps --------------------------------------------------------------
    def jump(self, state, k: int) -> np.ndarray:
        """original/mrg8.cpp semantics: J = prod A^(2^i), state <- J state."""
        st = _st(state)
        self.lib.orc_jump_ahead(_ptr(st), _ptr(self.tab), C.c_uint64(k))
        return st

    def jump_bits(self, state, bits) -> np.ndarray:
        st = _st(state)
        b = np.zeros(200, dtype=np.int16)
        b[: len(bits)] = bits
        self.lib.orc_jump_ahead_bits(_ptr(st), _ptr(self.tab), _ptr(b))
        return st

    def jump_matvec(self, state, k: int) -> np.ndarray:
        """knl/mrg8.h semantics: per-bit matrix-vector products."""
        st = _st(state)
        out = np.zeros(8, dtype=np.uint32)
        self.lib.orc_jump_ahead_matvec(_ptr(st), _ptr(self.tab), C.c_uint64(k), _ptr(out))
        return out

    def jump_matrix(self, k: int) -> np.ndarray:
        """Row-major A^k (k < 2^64) as a (8, 8) array."""
        bits = np.array([(k >> i) & 1 for i in range(64)] + [0] * 136, dtype=np.int16)
        J = np.zeros(64, dtype=np.uint32)
        self.lib.orc_jump_calc(_ptr(self.tab), _ptr(bits), _ptr(J))
        return J.reshape(8, 8)

    def read_jump_matrix(self, path: str) -> np.ndarray:
        tab = np.zeros(247 * 64, dtype=np.uint32)
        rc = self.lib.orc_read_jump_matrix(path.encode(), _ptr(tab))
        if rc != 0:
            raise OSError(f"cannot parse {path} ({rc})")
        return tab


def reference_dir():
    """Directory of the reference's sources, or None: $MRG8_REFERENCE, else the
    directory that ``make -C oracle ref REF=...`` recorded in _ref/REFDIR."""
    env = os.environ.get("MRG8_REFERENCE")
    if env:
        return env if os.path.isdir(env) else None
    try:
        with open(os.path.join(REF_DIR, "REFDIR")) as f:
            d = f.read().strip()
    except OSError:
        return None
    return d if d and os.path.isdir(d) else None


class RefLib:
    """One flavour of the reference compiled from its own sources."""

    FLAVOURS = ("original", "cudahost", "knl")

    def __init__(self, flavour: str, refdir: str):
        path = os.path.join(REF_DIR, f"libmrg8_ref_{flavour}.so")
        if not os.path.exists(path):
            raise FileNotFoundError(path)
        lib = C.CDLL(path)
        lib.ref_init.argtypes = [C.c_char_p]
        lib.ref_init.restype = C.c_int
        sub = {"original": "original", "cudahost": "cuda", "knl": "knl"}[flavour]
        rc = lib.ref_init(os.path.join(refdir, sub).encode())
        if rc != 0:
            raise OSError(f"ref_init({flavour}) failed: {rc}")
        lib.ref_seed.argtypes = [C.c_uint32, C.c_void_p]
        lib.ref_randint.argtypes = [C.c_void_p, C.c_void_p, C.c_int, C.c_void_p]
        lib.ref_rand.argtypes = [C.c_void_p, C.c_void_p, C.c_int, C.c_void_p]
        lib.ref_randint1.argtypes = [C.c_void_p, C.c_void_p]
        lib.ref_randint1.restype = C.c_uint32
        lib.ref_rand1.argtypes = [C.c_void_p, C.c_void_p]
        lib.ref_rand1.restype = C.c_double
        lib.ref_jump.argtypes = [C.c_void_p, C.c_uint64, C.c_void_p]
        lib.ref_jump_bits.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p]
        if flavour != "original":
            lib.ref_mrg8dnz2.argtypes = [C.c_void_p, C.c_void_p, C.c_int, C.c_void_p]
        if flavour == "knl":
            lib.ref_rand_tp.argtypes = [C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_void_p]
        self.lib = lib
        self.flavour = flavour

    def seed(self, seed: int) -> np.ndarray:
        st = np.zeros(8, dtype=np.uint32)
        self.lib.ref_seed(C.c_uint32(seed & 0xFFFFFFFF), _ptr(st))
        return st

    def randint(self, state, n: int):
        st, end = _st(state), np.zeros(8, dtype=np.uint32)
        out = np.empty(n, dtype=np.uint32)
        self.lib.ref_randint(_ptr(st), _ptr(out), n, _ptr(end))
        return out, end

    def rand(self, state, n: int):
        st, end = _st(state), np.zeros(8, dtype=np.uint32)
        out = np.empty(n, dtype=np.float64)
        self.lib.ref_rand(_ptr(st), _ptr(out), n, _ptr(end))
        return out, end

    def randint1(self, state):
        st, end = _st(state), np.zeros(8, dtype=np.uint32)
        return int(self.lib.ref_randint1(_ptr(st), _ptr(end))), end

    def rand1(self, state):
        st, end = _st(state), np.zeros(8, dtype=np.uint32)
        return float(self.lib.ref_rand1(_ptr(st), _ptr(end))), end

    def jump(self, state, k: int) -> np.ndarray:
        st, out = _st(state), np.zeros(8, dtype=np.uint32)
        self.lib.ref_jump(_ptr(st), C.c_uint64(k), _ptr(out))
        return out

    def jump_bits(self, state, bits) -> np.ndarray:
        st, out = _st(state), np.zeros(8, dtype=np.uint32)
        b = np.zeros(200, dtype=np.int16)
        b[: len(bits)] = bits
        self.lib.ref_jump_bits(_ptr(st), _ptr(b), _ptr(out))
        return out

    def mrg8dnz2(self, state, n: int):
        st, end = _st(state), np.zeros(8, dtype=np.uint32)
        out = np.empty(n, dtype=np.float64)
        self.lib.ref_mrg8dnz2(_ptr(st), _ptr(out), n, _ptr(end))
        return out, end

    def rand_tp(self, state, n: int, nthreads: int):
        st, end = _st(state), np.zeros(8, dtype=np.uint32)
        out = np.empty(n, dtype=np.float64)
        self.lib.ref_rand_tp(_ptr(st), _ptr(out), n, nthreads, _ptr(end))
        return out, end
