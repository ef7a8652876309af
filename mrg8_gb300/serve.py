"""Serving: device-resident generators and continuous batching of draw
requests (the mrg8g_server_* entry points of include/mrg8g.h)."""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib
from ._lib import check

_ELEM = {_lib.U32: (4, np.uint32), _lib.F64_ORIGINAL: (8, np.float64), _lib.F64_SHIFTED: (8, np.float64),
         _lib.F32_ORIGINAL: (4, np.float32), _lib.F32_SHIFTED: (4, np.float32)}


class Server:
    """A scheduler thread admits requests first-in first-out against a device
    output arena of ``budget_bytes`` and batches them into the persistent
    batch kernel on ``inflight`` streams."""

    def __init__(self, budget_bytes: int = 16 << 30, max_batch: int = 1024, inflight: int = 3,
                 max_generators: int = 65536, tile_rows: int = 0, threads: int = 0, spin_us: int = 0):
        self._lib = _lib.load()
        cfg = _lib.ServerConfig(budget_bytes, max_batch, inflight, max_generators, tile_rows, threads, spin_us)
        h = C.c_void_p()
        check(self._lib.mrg8g_server_create(C.byref(cfg), C.byref(h)))
        self._h = h

    def add_generator(self, state) -> int:
        st = np.ascontiguousarray(np.asarray(state, dtype=np.uint32))
        slot = C.c_uint32()
        check(self._lib.mrg8g_server_add_generator(self._h, st.ctypes.data, C.byref(slot)))
        return slot.value

    def generator_state(self, slot: int) -> np.ndarray:
        st = np.zeros(8, dtype=np.uint32)
        check(self._lib.mrg8g_server_generator_state(self._h, slot, st.ctypes.data))
        return st

    def submit(self, n: int, kind: int, seed: int = 0, offset: int = 0, generator: int | None = None,
               tag: int = 0) -> int:
        r = _lib.Request(_lib.NO_GENERATOR if generator is None else generator, seed & 0xFFFFFFFF, offset, n,
                         kind, 0, tag)
        t = C.c_uint64()
        check(self._lib.mrg8g_server_submit(self._h, C.byref(r), C.byref(t)))
        return t.value

    def poll(self, max_items: int = 256, timeout_us: int = 1000) -> list[dict]:
        buf = (_lib.Completion * max_items)()
        cnt = C.c_uint32()
        check(self._lib.mrg8g_server_poll(self._h, buf, max_items, C.byref(cnt), timeout_us))
        return [{"ticket": c.ticket, "tag": c.tag, "out": c.out, "n": c.n, "kind": c.kind, "status": c.status,
                 "t_submit": c.t_submit, "t_admit": c.t_admit, "t_done": c.t_done} for c in buf[:cnt.value]]

    def read(self, completion: dict) -> np.ndarray:
        size, dt = _ELEM[completion["kind"]]
        out = np.empty(completion["n"], dtype=dt)
        check(self._lib.mrg8g_server_read(self._h, completion["ticket"], out.ctypes.data, out.nbytes))
        return out

    def release(self, ticket: int) -> None:
        check(self._lib.mrg8g_server_release(self._h, ticket))

    def stats(self) -> dict:
        st = _lib.ServerStats()
        check(self._lib.mrg8g_server_get_stats(self._h, C.byref(st)))
        return {f: getattr(st, f) for f, _ in _lib.ServerStats._fields_ if f != "reserved"}

    def loadtest(self, rate: float, duration_s: float, n_min: int = 1 << 8, n_max: int = 1 << 26,
                 offset_max: int = 1 << 48, kinds_mask: int = 0b10111, hold_us: float = 0.0,
                 rng_seed: int = 1) -> dict:
        cfg = _lib.LoadtestConfig(rate, duration_s, hold_us, n_min, n_max, offset_max, rng_seed, kinds_mask, 0)
        res = _lib.LoadtestResult()
        check(self._lib.mrg8g_server_loadtest(self._h, C.byref(cfg), C.byref(res)))
        return {f: getattr(res, f) for f, _ in _lib.LoadtestResult._fields_}

    def close(self) -> None:
        if getattr(self, "_h", None):
            self._lib.mrg8g_server_destroy(self._h)
            self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):  # pragma: no cover
        try:
            self.close()
        except Exception:
            pass
