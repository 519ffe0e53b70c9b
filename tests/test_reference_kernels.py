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


def open_cases():
    with open(os.path.join(HERE, "golden", "reference_basefold.json")) as f:
        return json.load(f)["basefold_open_ref"]["cases"]


def case_inputs(case):
    if "evals" in case:
        ev = np.array(case["evals"], np.uint64)
    else:
        ev, _ = SI.c2_inputs(case["num_vars"])
    return ev, np.array(case["point"], np.uint64).reshape(-1, 2)


@pytest.mark.parametrize("case", open_cases(), ids=lambda c: c["name"])
def test_oracle_open_equals_reference_kernels(case):
    """The oracle's opening equals the one made by the reference's kernels, including the exact
    inputs of the reference's GPU-against-CPU opening test."""
    n, lr, q = case["num_vars"], case["log_rate"], case["num_queries"]
    ev, pt = case_inputs(case)
    assert sha(ev) == case["evals_sha256"]
    O.set_threads(os.cpu_count() or 1)
    try:
        c = O.basefold_commit(ev, lr)
        assert [int(x) for x in c["root"]] == case["root"]
        t = O.Transcript(case["label"].encode())
        if case["u64_after_label"] is not None:
            t.append_u64(b"", case["u64_after_label"])
        table = O.basefold_table(case["table_vars"], lr, case["table_vars"], case["table_seed"])
        proof = O.basefold_open_ext2(c, pt, table, t, q)
    finally:
        O.set_threads(1)
    assert proof.size == case["proof_len"]
    assert [int(x) for x in proof[:len(case["proof_head"])]] == case["proof_head"]
    assert sha(proof) == case["proof_sha256"]
    if "proof" in case:
        assert [int(x) for x in proof] == case["proof"]
    # and the restated verifier accepts it
    t = O.Transcript(case["label"].encode())
    if case["u64_after_label"] is not None:
        t.append_u64(b"", case["u64_after_label"])
    assert O.basefold_verify_ext2(c["root"], n, lr, pt, proof, q, table, t)


@pytest.mark.parametrize("n,lr,q,tv", [(2, 1, 1, 2), (3, 2, 5, 5), (5, 1, 34, 5), (7, 3, 8, 9), (9, 2, 20, 9)])
def test_reference_kernels_live_open(ref_lib, n, lr, q, tv):
    rng = np.random.default_rng(7000 + n)
    ev = rng.integers(0, O.P, size=1 << n, dtype=np.uint64)
    pt = rng.integers(0, O.P, size=(n, 2), dtype=np.uint64)
    table = O.basefold_table(tv, lr, tv, 5)
    rc = O.ref_basefold_commit(ev, lr)
    oc = O.basefold_commit(ev, lr)
    assert np.array_equal(rc["root"], oc["root"])
    want = O.basefold_open_ext2(oc, pt, table, O.Transcript(b"live"), q)
    got = O.ref_basefold_open_ext2(rc, pt, table, O.Transcript(b"live"), q)
    assert np.array_equal(got, want)


def sumcheck_cases():
    with open(os.path.join(HERE, "golden", "reference_basefold.json")) as f:
        return json.load(f)["sumcheck_ref"]["cases"]


@pytest.mark.parametrize("case", sumcheck_cases(), ids=lambda c: c["name"])
def test_oracle_sumcheck_equals_reference_kernels(case):
    d, n = case["degree"], case["num_vars"]
    polys = SI.field_elems(case["seed"], d << n).reshape(d, 1 << n)
    assert sha(polys) == case["polys_sha256"]
    r = O.sumcheck_prove_ext2(O.Transcript(case["label"].encode()), polys)
    for k in ("round_messages", "challenges", "final_evals", "final_eval"):
        assert [int(x) for x in np.asarray(r[k]).reshape(-1)] == case[k], k


@pytest.mark.parametrize("d,n", [(1, 1), (2, 9), (3, 7), (5, 4), (8, 3)])
def test_reference_kernels_live_sumcheck(ref_lib, d, n):
    polys = np.random.default_rng(40 + d * n).integers(0, O.P, size=(d, 1 << n), dtype=np.uint64)
    a = O.ref_sumcheck_prove_ext2(O.Transcript(b"live"), polys)
    b = O.sumcheck_prove_ext2(O.Transcript(b"live"), polys)
    for k in a:
        assert np.array_equal(a[k], b[k]), k
