"""Python mirror of the reference's generator classes over libmrg8g.so.

``MRG8`` mirrors ``class mrg8`` (original/mrg8.h:21-56, cuda/mrg8.h:23-79)
and ``MRG8Cuda`` mirrors ``class mrg8_cuda`` (cuda/mrg8_cuda.h:20-45): same
method names, argument meaning and state conventions (get_state returns
S[n-1] .. S[n-8], newest first).  Arrays may be CUDA torch tensors (device
path, stream-ordered on torch's current stream) or host numpy arrays / CPU
tensors (generated on the GPU and copied back).  Every value comes from the
CUDA kernels; there is no CPU fallback.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib
from ._lib import (F32_ORIGINAL, F32_SHIFTED, F64_ORIGINAL, F64_SHIFTED, ORIGINAL, SHIFTED, U32,
                   check)

try:  # torch is optional for host-only use
    import torch
except Exception:  # pragma: no cover
    torch = None

P = 2147483647
MAX_RND = 2147483646

_KIND_BYTES = {U32: 4, F64_ORIGINAL: 8, F64_SHIFTED: 8, F32_ORIGINAL: 4, F32_SHIFTED: 4}


def _kind(family: str, scaling: int) -> int:
    if scaling not in (ORIGINAL, SHIFTED):
        raise ValueError(f"scaling must be ORIGINAL (0) or SHIFTED (1), got {scaling}")
    if family == "f64":
        return F64_SHIFTED if scaling else F64_ORIGINAL
    return F32_SHIFTED if scaling else F32_ORIGINAL


def _target(arr, kind: int, n):
    """(pointer, element count, is_device, stream) for an output array."""
    if kind not in _KIND_BYTES:
        raise ValueError(f"unknown output kind {kind}")
    esize = _KIND_BYTES[kind]
    if torch is not None and isinstance(arr, torch.Tensor):
        if not arr.is_contiguous():
            raise ValueError("output tensor must be contiguous")
        if arr.element_size() != esize:
            raise TypeError(f"output tensor has {arr.element_size()}-byte elements, need {esize}")
        if kind != U32 and not arr.is_floating_point():
            raise TypeError("uniform outputs need a floating-point tensor")
        count = arr.numel()
        if n is None:
            n = count
        if n > count:
            raise ValueError(f"n = {n} exceeds the tensor size {count}")
        if arr.is_cuda:
            with torch.cuda.device(arr.device):
                stream = torch.cuda.current_stream(arr.device).cuda_stream
            return arr.data_ptr(), n, True, stream, arr.device
        return arr.data_ptr(), n, False, None, None
    a = arr
    if not isinstance(a, np.ndarray) or not a.flags.c_contiguous:
        raise TypeError("output must be a contiguous numpy array or torch tensor")
    if a.dtype.itemsize != esize:
        raise TypeError(f"output array has {a.dtype.itemsize}-byte elements, need {esize}")
    if n is None:
        n = a.size
    if n > a.size:
        raise ValueError(f"n = {n} exceeds the array size {a.size}")
    return a.ctypes.data, n, False, None, None


def _state_arr(st) -> np.ndarray:
    a = np.ascontiguousarray(np.asarray(st, dtype=np.uint64))
    if a.shape != (8,):
        raise ValueError("a state has 8 words")
    if (a >> np.uint64(32)).any():
        raise ValueError("state words are 32-bit")
    return a.astype(np.uint32)


def _bits200(bits) -> np.ndarray:
    b = np.zeros(200, dtype=np.int16)
    src = np.asarray(bits, dtype=np.int16)
    if src.size > 200:
        raise ValueError("at most 200 bits")
    b[: src.size] = src != 0
    return b


class MRG8:
    """The reference's ``mrg8`` class (original/mrg8.h:21-56)."""

    MAX_RND = MAX_RND
    #: scaling of rand()/mrg8dnz2 in the class this mirrors
    #: (original/mrg8.cpp:231-237 and cuda/mrg8.cpp:268-271: ORIGINAL).
    RAND_SCALING = ORIGINAL

    def __init__(self, seed_val: int = 0):
        self._lib = _lib.load()
        h = C.c_void_p()
        check(self._lib.mrg8g_create(C.c_uint32(seed_val & 0xFFFFFFFF), C.byref(h)))
        self._h = h

    def close(self) -> None:
        if getattr(self, "_h", None):
            self._lib.mrg8g_destroy(self._h)
            self._h = None

    def __del__(self):  # pragma: no cover - interpreter shutdown order
        try:
            self.close()
        except Exception:
            pass

    @property
    def handle(self) -> C.c_void_p:
        return self._h

    # ---------------------------------------------------------- state
    def seed_init(self, seed_val: int) -> None:
        check(self._lib.mrg8g_seed_init(self._h, C.c_uint32(seed_val & 0xFFFFFFFF)))

    def get_state(self, st=None) -> np.ndarray:
        out = np.zeros(8, dtype=np.uint32)
        check(self._lib.mrg8g_get_state(self._h, out.ctypes.data))
        if st is not None:
            st[:8] = out
        return out

    def set_state(self, st) -> None:
        a = _state_arr(st)
        check(self._lib.mrg8g_set_state(self._h, a.ctypes.data))

    def print_state(self) -> None:
        s = self.get_state()
        print("(S[n-1], S[n-2], ..., S[n-8])= (" + ", ".join(f"{int(v):>10d}" for v in s[:7])
              + f", {int(s[7])})")

    # ---------------------------------------------------------- jumps
    def jump_ahead(self, jump_val, new_state=None):
        """jump_ahead(k) advances the stream (original/mrg8.cpp:125-129);
        jump_ahead(k, new_state) writes the jumped state and leaves this one
        (cuda/mrg8.cpp:145-150).  k may be an int below 2^200 or a sequence
        of 200 bits with the LSB first (original/mrg8.cpp:104-122)."""
        if isinstance(jump_val, (int, np.integer)) and 0 <= int(jump_val) < (1 << 64):
            k = int(jump_val)
            if new_state is None:
                check(self._lib.mrg8g_jump_ahead(self._h, C.c_uint64(k)))
                return None
            out = np.zeros(8, dtype=np.uint32)
            check(self._lib.mrg8g_jump_state(self._h, C.c_uint64(k), out.ctypes.data))
        else:
            if isinstance(jump_val, (int, np.integer)):
                k = int(jump_val)
                if k < 0 or k >= (1 << 200):
                    raise ValueError("jump distance must lie in [0, 2^200)")
                bits = _bits200([(k >> i) & 1 for i in range(200)])
            else:
                bits = _bits200(jump_val)
            if new_state is None:
                check(self._lib.mrg8g_jump_ahead_bits(self._h, bits.ctypes.data))
                return None
            out = np.zeros(8, dtype=np.uint32)
            check(self._lib.mrg8g_jump_state_bits(self._h, bits.ctypes.data, out.ctypes.data))
        new_state[:8] = out
        return new_state

    # ---------------------------------------------------------- generation
    def _generate(self, arr, n, kind: int) -> None:
        ptr, n, dev, stream, device = _target(arr, kind, n)
        if n == 0:
            return
        if dev:
            with torch.cuda.device(device):
                check(self._lib.mrg8g_generate(self._h, C.c_void_p(ptr), C.c_uint64(n), kind,
                                               C.c_void_p(stream)))
        else:
            check(self._lib.mrg8g_generate_host(self._h, C.c_void_p(ptr), C.c_uint64(n), kind))

    def randint(self, iran=None, n=None):
        """randint(iran, n) fills iran with the next n values in [1, 2^31-1]
        (original/mrg8.cpp:197-222); randint() returns one value."""
        if iran is None:
            one = np.zeros(1, dtype=np.uint32)
            self._generate(one, 1, U32)
            return int(one[0])
        self._generate(iran, n, U32)
        return iran

    def rand(self, fran=None, n=None, scaling=None):
        """rand(fran, n) fills fran with the next n fp64 uniforms
        (original/mrg8.cpp:231-239); rand() returns one."""
        kind = _kind("f64", self.RAND_SCALING if scaling is None else scaling)
        if fran is None:
            one = np.zeros(1, dtype=np.float64)
            self._generate(one, 1, kind)
            return float(one[0])
        self._generate(fran, n, kind)
        return fran

    def __call__(self):
        return self.rand()

    def rand_f32(self, fran, n=None, scaling=None):
        """fp32 uniforms, (float) of the fp64 values."""
        self._generate(fran, n, _kind("f32", self.RAND_SCALING if scaling is None else scaling))
        return fran

    def mrg8dnz2(self, ran, n=None, scaling=None):
        """cuda/mrg8.cpp:290-339: the same values as rand().  The default is
        ORIGINAL scaling (S * rnorm), as the reference's cuda/ and original/
        classes; scaling=SHIFTED gives (S - 1) * rnorm, as the reference's KNL
        class (knl/mrg8.h:387-436)."""
        return self.rand(ran, n, scaling)


class MRG8Cuda(MRG8):
    """The reference's ``mrg8_cuda`` class (cuda/mrg8_cuda.h:20-45)."""

    @staticmethod
    def _check_launch(BS, TNUM):
        if BS is not None and (BS < 32 or BS > 1024 or BS % 32):
            raise ValueError(f"BS = {BS}: block size must be a multiple of 32 in [32, 1024]")
        if TNUM is not None and TNUM < 32:
            raise ValueError(f"TNUM = {TNUM}: need at least one warp")

    def mrg8_outer_32(self, d_ran, n=None, *launch):
        """mrg8_outer_32(d_ran, n[, TNUM]) / (d_ran, n, BS, TNUM): the next n
        SHIFTED fp64 uniforms into device memory (cuda/mrg8_cuda.cu:414-436).
        BS/TNUM only shaped the reference's launch; they do not change the
        values and the launch here is chosen for the GPU."""
        if len(launch) == 1:
            self._check_launch(None, launch[0])
        elif len(launch) == 2:
            self._check_launch(launch[0], launch[1])
        elif launch:
            raise TypeError("mrg8_outer_32(d_ran, n[, TNUM]) or (d_ran, n, BS, TNUM)")
        self._generate(d_ran, n, F64_SHIFTED)
        return d_ran

    def mrg8_inner(self, d_ran, n=None, TNUM=None):
        """cuda/mrg8_cuda.cu:402-412: same stream and scaling as mrg8_outer_32."""
        self._check_launch(None, TNUM)
        self._generate(d_ran, n, F64_SHIFTED)
        return d_ran

    def state_cpy_DtH(self) -> None:
        """cuda/mrg8_cuda.cu:72-79.  The state here is always current."""
        return None


def convert(d_in, d_out, scaling: int = ORIGINAL) -> None:
    """Uniforms from raw stream values S in [1, 2^31-1] (device tensors)."""
    lib = _lib.load()
    fam = "f64" if d_out.element_size() == 8 else "f32"
    kind = _kind(fam, scaling)
    n = d_in.numel()
    if d_out.numel() < n:
        raise ValueError("output too small")
    stream = torch.cuda.current_stream(d_in.device).cuda_stream
    with torch.cuda.device(d_in.device):
        check(lib.mrg8g_convert(C.c_void_p(d_in.data_ptr()), C.c_void_p(d_out.data_ptr()), C.c_uint64(n),
                                kind, C.c_void_p(stream)))


def jump_states(state, d_offsets) -> "torch.Tensor":
    """Device batch of jumps: row i = state advanced by d_offsets[i] outputs."""
    lib = _lib.load()
    st = _state_arr(state)
    if d_offsets.dtype not in (torch.int64, torch.uint64) or not d_offsets.is_contiguous():
        raise TypeError("offsets must be a contiguous 64-bit tensor")
    count = d_offsets.numel()
    out = torch.empty((count, 8), dtype=torch.int32, device=d_offsets.device)
    stream = torch.cuda.current_stream(d_offsets.device).cuda_stream
    with torch.cuda.device(d_offsets.device):
        check(lib.mrg8g_jump_states(st.ctypes.data, C.c_void_p(d_offsets.data_ptr()),
                                    C.c_void_p(out.data_ptr()), C.c_uint64(count), C.c_void_p(stream)))
    return out


class Batch:
    """Many independent generator instances in one persistent launch.

    ``instances`` is a sequence of ``(state, offset, out, kind)`` tuples (or
    dicts with those keys): ``state`` the 8-word state (``seed_state(seed)``
    for a seed), ``offset`` the outputs skipped first, ``out`` a contiguous
    CUDA tensor receiving ``out.numel()`` outputs (or ``n`` given explicitly
    as a fifth tuple item / dict key), ``kind`` one of U32, F64_*, F32_*.
    Each instance receives exactly the values of its own sequential stream.
    """

    def __init__(self, instances, tile_rows: int = 0, threads: int = 0, blocks_per_sm: int = 0,
                 use_graph: bool = True, tiling: int = 0):
        self._lib = _lib.load()
        items = []
        self._keep = []
        device = None
        for it in instances:
            if isinstance(it, dict):
                state, offset, out, kind, n = it["state"], it.get("offset", 0), it["out"], it["kind"], it.get("n")
            else:
                state, offset, out, kind = it[:4]
                n = it[4] if len(it) > 4 else None
            ptr, n, dev, _, dv = _target(out, kind, n)
            if not dev:
                raise TypeError("batch outputs must be CUDA tensors")
            device = device or dv
            inst = _lib.Instance()
            inst.state[:] = [int(v) for v in _state_arr(state)]
            inst.offset, inst.n, inst.out, inst.kind, inst.reserved = int(offset), int(n), ptr, int(kind), 0
            items.append(inst)
            self._keep.append(out)
        arr = (_lib.Instance * max(len(items), 1))(*items)
        self._arr, self._count = arr, len(items)
        cfg = _lib.BatchConfig(tile_rows, threads, blocks_per_sm, 1 if use_graph else 0, tiling)
        self.device = device
        h = C.c_void_p()
        with torch.cuda.device(device or torch.cuda.current_device()):
            check(self._lib.mrg8g_batch_create(arr, C.c_uint64(len(items)), C.byref(cfg), C.byref(h)))
        self._h = h

    def launch_each(self, stream=None) -> None:
        """The per-instance path: one bulk-kernel launch per instance."""
        with torch.cuda.device(self.device or torch.cuda.current_device()):
            s = (stream or torch.cuda.current_stream()).cuda_stream
            check(self._lib.mrg8g_generate_each(self._arr, C.c_uint64(self._count), C.c_void_p(s)))

    def launch(self, stream=None) -> None:
        """Enqueue the whole batch (one graph launch) on torch's current
        stream or the given one."""
        with torch.cuda.device(self.device or torch.cuda.current_device()):
            s = (stream or torch.cuda.current_stream()).cuda_stream
            check(self._lib.mrg8g_batch_launch(self._h, C.c_void_p(s)))

    def autotune(self) -> dict:
        with torch.cuda.device(self.device or torch.cuda.current_device()):
            cfg = _lib.BatchConfig()
            s = torch.cuda.current_stream().cuda_stream
            check(self._lib.mrg8g_batch_autotune(self._h, C.c_void_p(s), C.byref(cfg)))
        return {"tile_rows": cfg.tile_rows, "threads": cfg.threads, "blocks_per_sm": cfg.blocks_per_sm,
                "use_graph": cfg.use_graph, "tiling": cfg.tiling}

    @property
    def config(self) -> dict:
        cfg = _lib.BatchConfig()
        check(self._lib.mrg8g_batch_get_config(self._h, C.byref(cfg)))
        return {"tile_rows": cfg.tile_rows, "threads": cfg.threads, "blocks_per_sm": cfg.blocks_per_sm,
                "use_graph": cfg.use_graph, "tiling": cfg.tiling}

    def set_config(self, **kw) -> dict:
        """Change the launch shape (keys of ``config``; the others are kept)."""
        cur = self.config
        unknown = set(kw) - set(cur)
        if unknown:
            raise ValueError(f"unknown batch config keys {sorted(unknown)}")
        cur.update(kw)
        cfg = _lib.BatchConfig(cur["tile_rows"], cur["threads"], cur["blocks_per_sm"], 1 if cur["use_graph"] else 0,
                               cur["tiling"])
        check(self._lib.mrg8g_batch_set_config(self._h, C.byref(cfg)))
        return self.config

    def stats(self) -> dict:
        t, o, b = C.c_uint64(), C.c_uint64(), C.c_uint64()
        check(self._lib.mrg8g_batch_stats(self._h, C.byref(t), C.byref(o), C.byref(b)))
        return {"tiles": t.value, "outputs": o.value, "bytes": b.value}

    def close(self) -> None:
        if getattr(self, "_h", None):
            self._lib.mrg8g_batch_destroy(self._h)
            self._h = None

    def __del__(self):  # pragma: no cover
        try:
            self.close()
        except Exception:
            pass


def seed_state(seed: int) -> np.ndarray:
    """The state mcg64ni seeds from `seed` (original/mrg8.cpp:180-194)."""
    lib = _lib.load()
    st = np.zeros(8, dtype=np.uint32)
    check(lib.mrg8g_seed_state(C.c_uint32(seed & 0xFFFFFFFF), st.ctypes.data))
    return st


def generate_from_state(state, offset: int, out, kind: int, n=None, stream=None) -> None:
    """One instance through the bulk kernel (the per-instance path)."""
    lib = _lib.load()
    ptr, n, dev, s, device = _target(out, kind, n)
    if not dev:
        raise TypeError("generate_from_state writes device tensors")
    st = _state_arr(state)
    with torch.cuda.device(device):
        s = (stream.cuda_stream if stream is not None else s)
        check(lib.mrg8g_generate_from_state(st.ctypes.data, C.c_uint64(offset), C.c_void_p(ptr), C.c_uint64(n),
                                            kind, C.c_void_p(s)))
