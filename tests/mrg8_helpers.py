"""Small exact helpers for the tests (Python integers, no library code)."""
import numpy as np

P = 2147483647
COEF = [1089656042, 1906537547, 1764115693, 1304127872, 189748160, 1984088114, 626062218, 1927846343]
_INV_A8 = pow(COEF[7], P - 2, P)


def step_back(st):
    """State one output earlier: (S[n],...,S[n-7]) -> (S[n-1],...,S[n-8])."""
    s = [int(v) for v in st]
    acc = s[0] - sum(COEF[k] * s[k + 1] for k in range(7))
    oldest = (acc % P) * _INV_A8 % P
    return s[1:] + [oldest if oldest else P]


def state_with_output(m: int, residue: int, rng) -> np.ndarray:
    """A state whose output at stream position m (0-based) has the given
    residue mod p (0 gives the representative p)."""
    after = [int(v) for v in rng.integers(1, P, 8)]
    after[0] = residue % P if residue % P else P
    st = after
    for _ in range(m + 1):
        st = step_back(st)
    return np.array(st, dtype=np.uint32)


def u32_view(t):
    """uint32 numpy view of a torch int32/uint32 tensor (moved to host)."""
    return t.detach().cpu().numpy().view(np.uint32)


def bits64(a):
    return np.asarray(a).view(np.uint64)
