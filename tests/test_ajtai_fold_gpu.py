"""Ajtai fold-tree operations of zk-torch-4 through the C ABI (almost-goldilocks-cuda-rs
ajtai_fold_witness_ffi, ajtai_multifold_*_ffi, ajtai_split_witness_ffi, ajtai_*fold_commitment_ffi)
against the oracle's numpy restatement of cuda_almost_goldilocks/ajtai.cuh:700-1260: the
SuperNeo shapes (50 binary + 13 ternary instances, challenges in {-1, 0, 1, 2}, r_0 = 1) and
general int8 challenges; split followed by the folds reconstructs the witness."""
import ctypes

import numpy as np
import pytest

import oracle as O

pytestmark = pytest.mark.gpu
Q = O.Q_AGL


_KEEP = []


@pytest.fixture(autouse=True)
def _release_buffers():
    """Buffers made by dev() live until the test ends (a temporary passed as dev(x).ptr would
    otherwise be freed, and its memory reused, before the kernel that reads it runs)."""
    yield
    _KEEP.clear()


def dev(a):
    from morpheus_gb300.memory import DeviceBuffer
    buf = DeviceBuffer.from_numpy(np.ascontiguousarray(a))
    _KEEP.append(buf)
    return buf


def masks(rng, shape, density=0.5):
    bits = rng.random(size=shape + (64,)) < density
    return (bits.astype(np.uint64) << np.arange(64, dtype=np.uint64)).sum(axis=-1, dtype=np.uint64)


def superneo_r(rng, m):
    r = rng.choice([-1, 0, 1, 2], size=(m, 64)).astype(np.int8)
    r[0] = 0
    r[0, 0] = 1  # binary[0] has weight 1
    return r


@pytest.mark.parametrize("nb,nt,n_ring,general", [(50, 13, 300, False), (1, 0, 7, False), (3, 2, 1000, True),
                                                  (0, 13, 64, False), (63, 0, 129, False)])
def test_multifold_mixed_and_tc_forms(gpu_lib, nb, nt, n_ring, general):
    from morpheus_gb300 import _native as N
    L = N.lib()
    rng = np.random.default_rng(nb * 100 + nt)
    zb = masks(rng, (nb, n_ring)) if nb else np.zeros((0, n_ring), np.uint64)
    pos = masks(rng, (nt, n_ring), 0.3) if nt else np.zeros((0, n_ring), np.uint64)
    neg = (masks(rng, (nt, n_ring), 0.3) & ~pos) if nt else np.zeros((0, n_ring), np.uint64)
    r = rng.integers(-128, 128, size=(nb + nt, 64)).astype(np.int8) if general else superneo_r(rng, nb + nt)
    want = O.ajtai_multifold_mixed(zb, pos, neg, r)
    one = np.zeros(1, np.uint64)
    d_zb, d_pos, d_neg, d_r = dev(zb if nb else one), dev(pos if nt else one), dev(neg if nt else one), dev(r)
    for k, fn in enumerate([lambda o: L.ajtai_multifold_mixed_witness_ffi(d_zb.ptr, d_pos.ptr, d_neg.ptr, d_r.ptr, o, nb, nt, n_ring, 256),
                            lambda o: L.ajtai_multifold_mixed_witness_tc_ffi(d_zb.ptr, d_pos.ptr, d_neg.ptr, d_r.ptr, o, nb, nt, n_ring),
                            lambda o: L.ajtai_multifold_mixed_witness_tc_fused_ffi(d_zb.ptr, d_pos.ptr, d_neg.ptr, d_r.ptr, o, nb, nt, n_ring)]):
        out = dev(np.zeros(n_ring * 64, np.int16))
        assert fn(out.ptr) == 0
        L.cuda_sync_mine()
        assert np.array_equal(out.to_numpy().reshape(n_ring, 64), want), k
    if nt == 0:
        out = dev(np.zeros(n_ring * 64, np.int16))
        assert L.ajtai_multifold_witness_ffi(d_zb.ptr, d_r.ptr, out.ptr, nb, n_ring, 1024) == 0
        L.cuda_sync_mine()
        assert np.array_equal(out.to_numpy().reshape(n_ring, 64), want)
        assert L.ajtai_multifold_witness_ffi(d_zb.ptr, d_r.ptr, out.ptr, nb, n_ring, 0) == -2


@pytest.mark.parametrize("n_ring", [1, 33, 4096])
def test_fold_witness(gpu_lib, n_ring):
    from morpheus_gb300 import _native as N
    L = N.lib()
    rng = np.random.default_rng(n_ring)
    z1, z2 = masks(rng, (n_ring,)), masks(rng, (n_ring,))
    r = rng.choice([-1, 0, 1, 2], size=64).astype(np.int8)
    out = dev(np.zeros(n_ring * 64, np.uint64))
    assert L.ajtai_fold_witness_ffi(dev(z1).ptr, dev(z2).ptr, r.ctypes.data, n_ring, 128, out.ptr) == 0
    L.cuda_sync_mine()
    assert np.array_equal(out.to_numpy().reshape(n_ring, 64), O.ajtai_fold_witness(z1, z2, r))
    assert L.ajtai_fold_witness_ffi(dev(z1).ptr, dev(z2).ptr, r.ctypes.data, n_ring, 100, out.ptr) == -3


@pytest.mark.parametrize("n_ring", [1, 100, 5000])
def test_split_witness_reconstructs(gpu_lib, n_ring):
    from morpheus_gb300 import _native as N
    L = N.lib()
    rng = np.random.default_rng(n_ring + 1)
    z = rng.integers(-8191, 8192, size=(n_ring, 64)).astype(np.int16)
    z[0, :4] = [0, -8191, 8191, -1]
    d_pos, d_neg = dev(np.zeros(13 * n_ring, np.uint64)), dev(np.zeros(13 * n_ring, np.uint64))
    assert L.ajtai_split_witness_ffi(dev(z).ptr, d_pos.ptr, d_neg.ptr, n_ring) == 0
    L.cuda_sync_mine()
    pos, neg = d_pos.to_numpy().reshape(13, n_ring), d_neg.to_numpy().reshape(13, n_ring)
    wp, wn = O.ajtai_split_witness(z)
    assert np.array_equal(pos, wp) and np.array_equal(neg, wn)
    assert not (pos & neg).any()
    # folding the 13 chunks with r_i = 2^i (constant polynomials) gives the witness back
    r = np.zeros((13, 64), np.int8)
    r[:, 0] = [1 << i if i < 7 else 0 for i in range(13)]  # int8 holds 2^0..2^6
    out = dev(np.zeros(n_ring * 64, np.int16))
    assert L.ajtai_multifold_mixed_witness_ffi(dev(np.zeros(1, np.uint64)).ptr, d_pos.ptr, d_neg.ptr, dev(r).ptr,
                                               out.ptr, 0, 13, n_ring, 64) == 0
    L.cuda_sync_mine()
    low = sum((1 << i) * (O.bits64(pos[i]) - O.bits64(neg[i])) for i in range(7))
    assert np.array_equal(out.to_numpy().reshape(n_ring, 64), low.astype(np.int16))


@pytest.mark.parametrize("m", [1, 13, 63])
def test_commitment_folds(gpu_lib, m):
    from morpheus_gb300 import _native as N
    L = N.lib()
    rng = np.random.default_rng(m)
    c = rng.integers(0, 2**64 - 1, size=(m, 42, 64), dtype=np.uint64)  # non-canonical words too
    r = superneo_r(rng, m) if m > 1 else rng.integers(-128, 128, size=(1, 64)).astype(np.int8)
    out = dev(np.zeros(42 * 64, np.uint64))
    assert L.ajtai_multifold_commitment_ffi(dev(c).ptr, dev(r).ptr, m, out.ptr) == 0
    L.cuda_sync_mine()
    assert np.array_equal(out.to_numpy().reshape(42, 64), O.ajtai_fold_commitments(None, list(c), r))
    c1 = rng.integers(0, Q, size=(42, 64), dtype=np.uint64)
    assert L.ajtai_fold_commitment_ffi(dev(c1).ptr, dev(c[0]).ptr, r[0].ctypes.data, out.ptr) == 0
    L.cuda_sync_mine()
    assert np.array_equal(out.to_numpy().reshape(42, 64), O.ajtai_fold_commitments(c1, [c[0]], r[:1]))
