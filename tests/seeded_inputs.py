"""Platform-independent seeded inputs for the configuration-size parity tests.

The fixtures in tests/golden/config_goldens.json are made in one place and checked on another
machine, so their inputs must not depend on the numpy version there: they come from a
splitmix64 stream computed here with plain uint64 arithmetic.
"""
import numpy as np

P = 0xFFFFFFFF00000001
_GAMMA = np.uint64(0x9E3779B97F4A7C15)
_M1 = np.uint64(0xBF58476D1CE4E5B9)
_M2 = np.uint64(0x94D049BB133111EB)


def splitmix64(seed, count):
    """count outputs of splitmix64 from state `seed` (outputs 1..count)."""
    with np.errstate(over="ignore"):
        z = np.uint64(seed) + _GAMMA * np.arange(1, count + 1, dtype=np.uint64)
        z = (z ^ (z >> np.uint64(30))) * _M1
        z = (z ^ (z >> np.uint64(27))) * _M2
        return z ^ (z >> np.uint64(31))


def field_elems(seed, count):
    """count Goldilocks elements in [0, p): splitmix64 outputs reduced mod p (bias 2^-32)."""
    return splitmix64(seed, count) % np.uint64(P)


# C1: two multilinear polynomials of 2^20 evaluations each, transcript label "bench"
C1 = {"num_vars": 20, "degree": 2, "seed": 0xC1, "label": b"bench"}
# C2: one polynomial of 2^22 evaluations, rate 1/2, 34 queries, table (22, 1, 22, seed 42),
# opened at an Ext2 point on the transcript "bf-open"
C2 = {"num_vars": 22, "log_rate": 1, "num_queries": 34, "table_seed": 42, "seed": 0xC2, "label": b"bf-open"}


def c1_polys():
    n, d = C1["num_vars"], C1["degree"]
    return field_elems(C1["seed"], d << n).reshape(d, 1 << n)


def c2_inputs(num_vars=None):
    """(evaluations, Ext2 point [n][2]) of the C2 configuration (or of num_vars variables)."""
    n = C2["num_vars"] if num_vars is None else num_vars
    v = field_elems(C2["seed"] + n, (1 << n) + 2 * n)
    return v[: 1 << n].copy(), v[1 << n:].reshape(n, 2).copy()
