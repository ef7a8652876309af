"""mrg8_gb300 -- GB300-native MRG8 generator (drop-in for kenmiura/mrg8's
mrg8 / mrg8_cuda path).

The compute path is libmrg8g.so (hand-written sm_103a kernels behind the C ABI
of include/mrg8g.h); this package loads it through ctypes and mirrors the
reference classes.  Build the library with ``python -m mrg8_gb300.build``.
"""
from ._lib import (F32_ORIGINAL, F32_SHIFTED, F64_ORIGINAL, F64_SHIFTED, ORIGINAL, SHIFTED, U32,
                   MRG8GError, load)
from .api import MAX_RND, MRG8, Batch, MRG8Cuda, P, convert, generate_from_state, jump_states, seed_state

__all__ = [
    "MRG8", "MRG8Cuda", "Batch", "MRG8GError", "load", "convert", "jump_states", "seed_state",
    "generate_from_state", "P", "MAX_RND",
    "ORIGINAL", "SHIFTED", "U32", "F64_ORIGINAL", "F64_SHIFTED", "F32_ORIGINAL", "F32_SHIFTED",
]
