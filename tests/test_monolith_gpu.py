"""Monolith-12 permutation and Merkle trees on the GPU against the oracle (pinned to the
reference's known-answer vector) on the reference's own test inputs and random trees."""
import numpy as np
import pytest

import oracle as O

pytestmark = pytest.mark.gpu
P = O.P


def _permute(state):
    from morpheus_gb300 import _native as N
    s = np.ascontiguousarray(state, np.uint64)
    out = np.zeros(12, np.uint64)
    N.check(N.lib().monolith_permute_test_ffi(s.ctypes.data, out.ctypes.data), "monolith_permute_test_ffi")
    return out


def test_permutation_kat_and_large_values(gpu_lib, golden):
    g = golden["monolith_kat"]
    assert [int(x) for x in _permute(np.array(g["input"], np.uint64))] == g["expected"]
    large = np.array(golden["monolith_tree_inputs"]["large_value_state"], np.uint64)
    assert np.array_equal(_permute(large), O.monolith_permute(large))
    rng = np.random.default_rng(12)
    for _ in range(8):
        s = rng.integers(0, 1 << 64, size=12, dtype=np.uint64)  # non-canonical words too
        assert np.array_equal(_permute(s), O.monolith_permute(s))


def _tree(cw, ext2):
    from morpheus_gb300 import _native as N
    from morpheus_gb300.memory import DeviceBuffer
    cw = np.ascontiguousarray(cw, np.uint64)
    leaves = cw.size // (4 if ext2 else 2)
    d_cw, d_tree = DeviceBuffer.from_numpy(cw), DeviceBuffer((2 * leaves - 1) * 4)
    fn = N.lib().monolith_merkle_tree_ext2_ffi if ext2 else N.lib().monolith_merkle_tree_gl_ffi
    N.check(fn(d_cw.ptr, d_tree.ptr, leaves), "monolith tree")
    return d_tree.to_numpy()


def test_trees_on_reference_test_codewords(gpu_lib, golden):
    g = golden["monolith_tree_inputs"]
    for cw in g["codewords"]:
        cw = np.array(cw, np.uint64)
        assert np.array_equal(_tree(cw, False), O.monolith_tree_gl(cw))
    e = np.array(g["ext2_codeword"], np.uint64)
    assert np.array_equal(_tree(e, True), O.monolith_tree_ext2(e))


@pytest.mark.parametrize("leaves", [1, 2, 64, 1 << 13])
def test_random_trees(gpu_lib, leaves):
    rng = np.random.default_rng(leaves)
    cw = rng.integers(0, P, size=2 * leaves, dtype=np.uint64)
    assert np.array_equal(_tree(cw, False), O.monolith_tree_gl(cw))
    e = rng.integers(0, P, size=4 * leaves, dtype=np.uint64)
    assert np.array_equal(_tree(e, True), O.monolith_tree_ext2(e))


def test_rejects_empty_tree(gpu_lib):
    from morpheus_gb300 import _native as N
    assert N.lib().monolith_merkle_tree_gl_ffi(None, None, 0) == -2
    assert N.lib().monolith_cuda_init() == 0
