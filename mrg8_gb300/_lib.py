"""ctypes binding of libmrg8g.so (the C ABI declared in include/mrg8g.h).

The library is built in-tree by ``mrg8_gb300.build``.  Loading fails loudly
when it is missing: there is no CPU fallback anywhere in this package.
"""
from __future__ import annotations

import ctypes as C
import os
import threading

from . import build as _build

LIB_PATH = _build.LIB

SUCCESS = 0
ERR_INVALID_ARGUMENT = -1
ERR_INVALID_STATE = -2
ERR_CUDA = -3
ERR_OUT_OF_MEMORY = -4
ERR_TIMEOUT = -5
ERR_BUDGET = -6
ERR_NOT_READY = -7

ORIGINAL, SHIFTED = 0, 1
U32, F64_ORIGINAL, F64_SHIFTED, F32_ORIGINAL, F32_SHIFTED = range(5)

_vp = C.c_void_p
_u32 = C.c_uint32
_u64 = C.c_uint64
_int = C.c_int

# name -> (restype, argtypes); every symbol declared in include/mrg8g.h.
SIGNATURES: dict[str, tuple] = {
    "mrg8g_version": (_int, []),
    "mrg8g_last_error": (C.c_char_p, []),
    "mrg8g_create": (_int, [_u32, _vp]),
    "mrg8g_destroy": (_int, [_vp]),
    "mrg8g_seed_init": (_int, [_vp, _u32]),
    "mrg8g_get_state": (_int, [_vp, _vp]),
    "mrg8g_set_state": (_int, [_vp, _vp]),
    "mrg8g_jump_ahead": (_int, [_vp, _u64]),
    "mrg8g_jump_ahead_bits": (_int, [_vp, _vp]),
    "mrg8g_jump_state": (_int, [_vp, _u64, _vp]),
    "mrg8g_jump_state_bits": (_int, [_vp, _vp, _vp]),
    "mrg8g_randint": (_int, [_vp, _vp, _u64, _vp]),
    "mrg8g_rand": (_int, [_vp, _vp, _u64, _int, _vp]),
    "mrg8g_rand_f32": (_int, [_vp, _vp, _u64, _int, _vp]),
    "mrg8g_generate": (_int, [_vp, _vp, _u64, _int, _vp]),
    "mrg8g_generate_host": (_int, [_vp, _vp, _u64, _int]),
    "mrg8g_convert": (_int, [_vp, _vp, _u64, _int, _vp]),
    "mrg8g_jump_states": (_int, [_vp, _vp, _vp, _u64, _vp]),
    "mrg8g_generate_from_state": (_int, [_vp, _u64, _vp, _u64, _int, _vp]),
    "mrg8g_write_jump_matrix": (_int, [C.c_char_p]),
    "mrg8g_verify_jump_matrix": (_int, [C.c_char_p, _vp]),
    "mrg8g_seed_state": (_int, [_u32, _vp]),
    "mrg8g_stream_sync": (_int, [_vp]),
    "mrg8g_tune_plain": (_int, [_int, _int, _int]),
    "mrg8g_get_plain_tuning": (_int, [_int, _vp, _vp]),
    "mrg8g_batch_create": (_int, [_vp, _u64, _vp, _vp]),
    "mrg8g_batch_launch": (_int, [_vp, _vp]),
    "mrg8g_batch_autotune": (_int, [_vp, _vp, _vp]),
    "mrg8g_batch_get_config": (_int, [_vp, _vp]),
    "mrg8g_batch_set_config": (_int, [_vp, _vp]),
    "mrg8g_batch_stats": (_int, [_vp, _vp, _vp, _vp]),
    "mrg8g_batch_destroy": (_int, [_vp]),
    "mrg8g_generate_each": (_int, [_vp, _u64, _vp]),
    "mrg8g_batch_generate_noalloc": (_int, [_vp, _u64, _vp]),
    "mrg8g_server_create": (_int, [_vp, _vp]),
    "mrg8g_server_add_generator": (_int, [_vp, _vp, _vp]),
    "mrg8g_server_generator_state": (_int, [_vp, _u32, _vp]),
    "mrg8g_server_submit": (_int, [_vp, _vp, _vp]),
    "mrg8g_server_poll": (_int, [_vp, _vp, _u32, _vp, _u32]),
    "mrg8g_server_read": (_int, [_vp, _u64, _vp, _u64]),
    "mrg8g_server_release": (_int, [_vp, _u64]),
    "mrg8g_server_get_stats": (_int, [_vp, _vp]),
    "mrg8g_server_destroy": (_int, [_vp]),
    "mrg8g_server_loadtest": (_int, [_vp, _vp, _vp]),
}


class Instance(C.Structure):
    """mrg8g_instance of include/mrg8g.h."""
    _fields_ = [("state", C.c_uint32 * 8), ("offset", C.c_uint64), ("n", C.c_uint64), ("out", C.c_void_p),
                ("kind", C.c_int32), ("reserved", C.c_int32)]


class ServerConfig(C.Structure):
    """mrg8g_server_config of include/mrg8g.h."""
    _fields_ = [("budget_bytes", C.c_uint64), ("max_batch", C.c_uint32), ("inflight", C.c_uint32),
                ("max_generators", C.c_uint32), ("tile_rows", C.c_int32), ("threads", C.c_int32),
                ("spin_us", C.c_int32)]


NO_GENERATOR = 0xFFFFFFFF


class Request(C.Structure):
    """mrg8g_request of include/mrg8g.h."""
    _fields_ = [("generator", C.c_uint32), ("seed", C.c_uint32), ("offset", C.c_uint64), ("n", C.c_uint64),
                ("kind", C.c_int32), ("reserved", C.c_int32), ("tag", C.c_uint64)]


class Completion(C.Structure):
    """mrg8g_completion of include/mrg8g.h."""
    _fields_ = [("ticket", C.c_uint64), ("tag", C.c_uint64), ("out", C.c_void_p), ("n", C.c_uint64),
                ("kind", C.c_int32), ("status", C.c_int32), ("t_submit", C.c_double), ("t_admit", C.c_double),
                ("t_done", C.c_double)]


class ServerStats(C.Structure):
    """mrg8g_server_stats of include/mrg8g.h."""
    _fields_ = [("submitted", C.c_uint64), ("completed", C.c_uint64), ("pending", C.c_uint64),
                ("launches", C.c_uint64), ("launched_requests", C.c_uint64), ("samples", C.c_uint64),
                ("bytes_in_use", C.c_uint64), ("peak_bytes", C.c_uint64), ("error", C.c_int32),
                ("reserved", C.c_int32), ("max_inflight", C.c_uint64), ("overlapped_launches", C.c_uint64),
                ("mean_batch", C.c_double), ("kernel_ns", C.c_uint64), ("kernel_launches", C.c_uint64)]


class LoadtestConfig(C.Structure):
    """mrg8g_loadtest_config of include/mrg8g.h."""
    _fields_ = [("rate", C.c_double), ("duration_s", C.c_double), ("hold_us", C.c_double), ("n_min", C.c_uint64),
                ("n_max", C.c_uint64), ("offset_max", C.c_uint64), ("rng_seed", C.c_uint64),
                ("kinds_mask", C.c_uint32), ("reserved", C.c_uint32)]


class LoadtestResult(C.Structure):
    """mrg8g_loadtest_result of include/mrg8g.h."""
    _fields_ = [("requests", C.c_uint64), ("samples", C.c_uint64), ("bytes", C.c_uint64), ("launches", C.c_uint64),
                ("peak_bytes", C.c_uint64), ("late_submits", C.c_uint64), ("wall_s", C.c_double),
                ("gsamples_per_s", C.c_double), ("mean_us", C.c_double), ("p50_us", C.c_double),
                ("p90_us", C.c_double), ("p99_us", C.c_double), ("max_us", C.c_double), ("mean_batch", C.c_double),
                ("max_inflight", C.c_uint64), ("overlapped_launches", C.c_uint64), ("mean_kernel_us", C.c_double)]


class BatchConfig(C.Structure):
    """mrg8g_batch_config of include/mrg8g.h."""
    _fields_ = [("tile_rows", C.c_int32), ("threads", C.c_int32), ("blocks_per_sm", C.c_int32),
                ("use_graph", C.c_int32), ("tiling", C.c_int32)]


class MRG8GError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"[{code}] {msg}")
        self.code = code


_lock = threading.Lock()
_lib = None


def load(build_if_missing: bool = False):
    """Load libmrg8g.so (optionally building it first)."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        if not os.path.exists(LIB_PATH):
            if not build_if_missing:
                raise OSError(
                    f"{LIB_PATH} is missing: build it with `python -m mrg8_gb300.build` "
                    "(this package has no CPU fallback)")
            _build.build()
        lib = C.CDLL(LIB_PATH)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        _lib = lib
        return lib


def check(rc: int) -> None:
    if rc != SUCCESS:
        msg = _lib.mrg8g_last_error().decode(errors="replace") if _lib is not None else ""
        raise MRG8GError(rc, msg)
