"""Regenerate tests/golden/mrg8_kat.json from the reference itself.

Runs kenmiura/mrg8 compiled from its own sources (``make -C oracle ref``
builds oracle/_ref/ from the reference tree) and records known answers: seed
states, stream prefixes and far positions, both fp64 scalings, jumps (64-bit
and 200-bit), mrg8dnz2, and digests of long runs.  Usage:

    make -C oracle ref REF=/path/to/mrg8
    python tests/golden/make_golden.py /path/to/mrg8
"""
from __future__ import annotations

import hashlib
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))
from oracle.pyoracle import RefLib  # noqa: E402

OUT = os.path.join(HERE, "mrg8_kat.json")


def hexf(a: np.ndarray) -> list[str]:
    return [f"{int(v):016x}" for v in np.asarray(a, dtype=np.float64).view(np.uint64)]


def digest(a: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def main(refdir: str) -> None:
    ro = RefLib("original", refdir)
    rc = RefLib("cudahost", refdir)
    rk = RefLib("knl", refdir)
    kat: dict = {"generated_by": "tests/golden/make_golden.py from the reference build in oracle/_ref"}

    seeds = [0, 1, 2, 13579, 97531, 2**31 - 1, 2**32 - 1, 123456789]
    kat["seed_states"] = {str(s): [int(v) for v in ro.seed(s)] for s in seeds}

    st = ro.seed(13579)
    n24 = 1 << 24
    ints, end = ro.randint(st, n24)
    kat["seed13579"] = {
        "randint_first64": [int(v) for v in ints[:64]],
        "randint_at": {str(i): int(ints[i]) for i in (1000, (1 << 20) - 1, (1 << 22) + 7, n24 - 1)},
        "state_after_2^24": [int(v) for v in end],
        "min_2^24": int(ints.min()),
        "max_2^24": int(ints.max()),
        "sum_2^24": int(ints.astype(np.uint64).sum()),
        "sha256_randint_2^24": digest(ints),
    }
    f_orig, _ = ro.rand(st, n24)
    kat["seed13579"]["rand_original_first16_bits"] = hexf(f_orig[:16])
    kat["seed13579"]["rand_original_at_2^24-1_bits"] = hexf(f_orig[-1:])[0]
    kat["seed13579"]["sha256_rand_original_2^24"] = digest(f_orig)
    f_sh, _ = rk.rand(st, n24)
    kat["seed13579"]["rand_shifted_first16_bits"] = hexf(f_sh[:16])
    kat["seed13579"]["sha256_rand_shifted_2^24"] = digest(f_sh)
    kat["seed13579"]["sha256_f32_original_2^24"] = digest(f_orig.astype(np.float32))
    kat["seed13579"]["sha256_f32_shifted_2^24"] = digest(f_sh.astype(np.float32))
    one, end1 = ro.randint1(st)
    kat["seed13579"]["randint_scalar"] = {"value": one, "state": [int(v) for v in end1]}
    r1, _ = ro.rand1(st)
    kat["seed13579"]["rand_scalar_bits"] = hexf(np.array([r1]))[0]

    # Jumps from the seeded state and from a state with a zero word and a p word.
    odd = st.copy()
    odd[2] = 0
    odd[5] = 2**31 - 1
    ks = [0, 1, 5, 7, 8, 9, 1000, 2**31 + 17, 2**40 + 3, 2**63 + 12345, 2**64 - 1]
    kat["jumps"] = []
    for base_name, base in (("seed13579", st), ("odd", odd)):
        for k in ks:
            kat["jumps"].append({"from": base_name, "state": [int(v) for v in base], "k": str(k),
                                 "original": [int(v) for v in ro.jump(base, k)],
                                 "knl": [int(v) for v in rk.jump(base, k)]})
    rng = np.random.default_rng(20240601)
    kat["jumps200"] = []
    for t in range(4):
        bits = [int(b) for b in rng.integers(0, 2, 200)]
        if t == 0:
            bits = [0] * 199 + [1]  # 2^199
        kat["jumps200"].append({"state": [int(v) for v in st], "bits": "".join(map(str, bits)),
                                "original": [int(v) for v in ro.jump_bits(st, bits)],
                                "cudahost": [int(v) for v in rc.jump_bits(st, bits)]})

    # Known-answer check of the advertised jump semantics: jump(k) then randint.
    j5 = ro.jump(st, 5)
    after, _ = ro.randint(j5, 8)
    kat["jump5_then_randint8"] = [int(v) for v in after]

    # mrg8dnz2: ORIGINAL (cuda/mrg8.cpp) and SHIFTED (knl/mrg8.h), block + remainder.
    d_o, e_o = rc.mrg8dnz2(st, 3000)
    d_s, e_s = rk.mrg8dnz2(st, 3000)
    kat["mrg8dnz2_3000"] = {"original_sha256": digest(d_o), "original_state": [int(v) for v in e_o],
                            "shifted_sha256": digest(d_s), "shifted_state": [int(v) for v in e_s],
                            "original_last4_bits": hexf(d_o[-4:]), "shifted_first4_bits": hexf(d_s[:4])}

    # The reference's jump table file, as numbers.
    tab = np.loadtxt(os.path.join(refdir, "original", "jump_matrix.txt"), dtype=np.uint64).reshape(-1)
    kat["jump_matrix_txt"] = {"count": int(tab.size), "sum": int(tab.sum()),
                              "sha256_u32": digest(tab.astype(np.uint32)),
                              "entries_0_16": [int(v) for v in tab[:16]],
                              "matrix246_first8": [int(v) for v in tab[246 * 64: 246 * 64 + 8]]}

    with open(OUT, "w") as f:
        json.dump(kat, f, indent=1)
    print("wrote", OUT)


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python tests/golden/make_golden.py <directory of the reference's sources>")
    main(sys.argv[1])
