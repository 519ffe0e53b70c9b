"""The oracle against the reference's own Basefold kernels.

tests/golden/reference_basefold.json holds commitments made by the reference's kernels
(cuda/basefold.cuh, and the Merkle kernels of goldilocks-cuda-rs/cuda/wrapper.cu) run on the host
by oracle/_ref/libbasefold_ref.so, on the platform-independent inputs of tests/seeded_inputs.py.
The oracle must reproduce each one.  Where the reference checkout was available to build
oracle/_ref, the same kernels are also compared with the oracle live on further shapes."""
import ctypes
import hashlib
import json
import os

import numpy as np
import pytest

import oracle as O
import seeded_inputs as SI

HERE = os.path.dirname(os.path.abspath(__file__))
REF_LIB = os.path.join(os.path.dirname(HERE), "oracle", "_ref", "libbasefold_ref.so")


def sha(a):
    return hashlib.sha256(np.ascontiguousarray(a, dtype="<u8").tobytes()).hexdigest()


def fixture_cases():
    with open(os.path.join(HERE, "golden", "reference_basefold.json")) as f:
        return json.load(f)["basefold_commit_ref"]["cases"]


@pytest.mark.parametrize("case", fixture_cases(), ids=lambda c: f"n{c['num_vars']}_lr{c['log_rate']}")
def test_oracle_commit_equals_reference_kernels(case):
    n, lr = case["num_vars"], case["log_rate"]
    ev, _ = SI.c2_inputs(n)
    assert sha(ev) == case["evals_sha256"]
    O.set_threads(os.cpu_count() or 1)
    try:
        c = O.basefold_commit(ev, lr)
    finally:
        O.set_threads(1)
    assert [int(x) for x in c["root"]] == case["root"]
    assert sha(c["codeword"]) == case["codeword_sha256"]
    assert sha(c["bh_evals"]) == case["bh_evals_sha256"]
    assert sha(c["tree"]) == case["tree_sha256"]
    if "codeword" in case:
        assert [int(x) for x in c["codeword"]] == case["codeword"]


@pytest.fixture(scope="module")
def ref_lib():
    if not os.path.exists(REF_LIB):
        pytest.skip("oracle/_ref/libbasefold_ref.so is built only where the reference checkout exists")
    R = ctypes.CDLL(REF_LIB)
    u = np.ctypeslib.ndpointer(dtype=np.uint64, flags="C_CONTIGUOUS")
    R.ref_bf_init()
    R.ref_basefold_commit.argtypes = [u, ctypes.c_int, ctypes.c_int, u, u, u, u]
    R.ref_merkle_tree_ext2.argtypes = [u, u, ctypes.c_int]
    return R


@pytest.mark.parametrize("n,lr", [(2, 1), (3, 2), (5, 1), (8, 3), (11, 2)])
def test_reference_kernels_live_commit(ref_lib, n, lr):
    rng = np.random.default_rng(1000 + 10 * n + lr)
    ev = rng.integers(0, O.P, size=1 << n, dtype=np.uint64)
    L = 1 << (n + lr)
    cw, bh = np.zeros(L, np.uint64), np.zeros(1 << n, np.uint64)
    tree, root = np.zeros((L - 1) * 4, np.uint64), np.zeros(4, np.uint64)
    ref_lib.ref_basefold_commit(ev, n, lr, cw, bh, tree, root)
    c = O.basefold_commit(ev, lr)
    P = np.uint64(O.P)
    assert np.array_equal(root % P, c["root"]) and np.array_equal(cw % P, c["codeword"])
    assert np.array_equal(bh % P, c["bh_evals"]) and np.array_equal(tree % P, c["tree"])


@pytest.mark.parametrize("leaves", [1, 2, 64, 1 << 10])
def test_reference_kernels_live_ext2_tree(ref_lib, leaves):
    rng = np.random.default_rng(leaves)
    cw = rng.integers(0, O.P, size=4 * leaves, dtype=np.uint64)
    tree = np.zeros((2 * leaves - 1) * 4, np.uint64)
    ref_lib.ref_merkle_tree_ext2(cw, tree, leaves)
    assert np.array_equal(tree % np.uint64(O.P), O.merkle_tree_ext2(cw))
