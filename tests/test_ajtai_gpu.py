"""Ajtai commitment on the GPU against the reference's own CPU code (golden vectors) and the oracle."""
import numpy as np
import pytest

import oracle as O

Q = O.Q_AGL
pytestmark = pytest.mark.gpu


def test_commit_wide_matches_reference(gpu_lib, golden):
    from morpheus_gb300 import ajtai
    g = golden["ajtai_commit_wide_ref"]
    c = ajtai.commit_wide(g["key"], np.array(g["z"], np.uint64), col_offset=g["col_offset"])
    assert [int(x) for x in c.reshape(-1)] == g["out"]


def test_commit_wide_binary_matches_reference(gpu_lib, golden):
    from morpheus_gb300 import ajtai
    g = golden["ajtai_commit_binary_ref"]
    bits = np.array([[(w >> l) & 1 for l in range(64)] for w in g["z_bits"]], np.uint64).reshape(-1)
    for chunk in (64, 4096):
        c = ajtai.commit_wide(g["key"], bits, chunk=chunk)
        assert [int(x) for x in c.reshape(-1)] == g["out"]


def test_commit_wide_random_vs_oracle(gpu_lib):
    from morpheus_gb300 import ajtai
    key = np.array([3, 1, 4, 1, 5, 9, 2, 6], np.uint32)
    z = np.random.default_rng(5).integers(0, Q, size=37 * 64, dtype=np.uint64)
    assert np.array_equal(ajtai.commit_wide(key, z, col_offset=11), O.ajtai_commit_wide(key, z, 11, 0, 42))


def test_commit_wide_rejects_unsupported_chunk(gpu_lib):
    """almost wrapper.cu:1203: a chunk outside {64, 128, 256, 1024, 4096} returns -3."""
    from morpheus_gb300 import ajtai
    from morpheus_gb300 import _native as N
    key = np.arange(8, dtype=np.uint32)
    z = np.ones(64, np.uint64)
    for chunk in (100, 512, 8192):
        with pytest.raises(RuntimeError, match="-3"):
            ajtai.commit_wide(key, z, chunk=chunk)
    for chunk in (0, -64, 100):
        assert N.lib().ajtai_commit_wide_ffi(None, None, 1, 0, chunk, None) == -3


def test_batched_matches_reference(gpu_lib, golden):
    from morpheus_gb300.ajtai import AjtaiKey
    g = golden["ajtai_commit_u8_ref"]
    k = AjtaiKey(g["key"], 0, g["rows"], g["N"])
    out = k.commit_u8_batched(np.array(g["z"], np.uint8).reshape(1, -1))
    assert [int(x) for x in out.reshape(-1)] == g["out"]


@pytest.mark.parametrize("n_ring,B,row_lo,rows", [(16, 3, 0, 16), (40, 5, 0, 16), (8, 130, 3, 2), (33, 1, 40, 2)])
def test_batched_vs_oracle(gpu_lib, n_ring, B, row_lo, rows):
    from morpheus_gb300.ajtai import AjtaiKey
    key = np.array([9, 8, 7, 6, 5, 4, 3, 2], np.uint32)
    z8 = np.random.default_rng(n_ring + B).integers(0, 256, size=(B, n_ring * 64), dtype=np.uint8)
    k = AjtaiKey(key, row_lo, rows, n_ring)
    out = k.commit_u8_batched(z8)
    pick = sorted({0, B - 1, B // 2})
    ref = O.ajtai_commit_u8_batch(key, z8[pick], row_lo=row_lo, nrows=rows)
    assert np.array_equal(out[pick], ref)


def test_batched_extremes_and_batch_invariance(gpu_lib):
    from morpheus_gb300.ajtai import AjtaiKey
    key = np.array([1, 2, 3, 4, 5, 6, 7, 8], np.uint32)
    n_ring = 32
    z = np.zeros((4, n_ring * 64), np.uint8)
    z[1] = 255
    z[2] = np.random.default_rng(1).integers(0, 256, size=n_ring * 64, dtype=np.uint8)
    z[3, ::3] = 255
    k = AjtaiKey(key, 0, 4, n_ring)
    out = k.commit_u8_batched(z)
    assert not out[0].any()
    ref = O.ajtai_commit_u8_batch(key, z, row_lo=0, nrows=4)
    assert np.array_equal(out, ref)
    # a witness's commitment does not depend on its batch position or companions
    out2 = k.commit_u8_batched(z[[2, 3, 1]])
    assert np.array_equal(out2, out[[2, 3, 1]])


def test_batched_equals_wide_rows(gpu_lib):
    from morpheus_gb300 import ajtai
    key = np.array([11, 22, 33, 44, 55, 66, 77, 88], np.uint32)
    n_ring = 16
    z8 = np.random.default_rng(2).integers(0, 256, size=(2, n_ring * 64), dtype=np.uint8)
    out = ajtai.AjtaiKey(key, 0, 42, n_ring).commit_u8_batched(z8)
    for b in range(2):
        assert np.array_equal(out[b], ajtai.commit_wide(key, z8[b].astype(np.uint64)))


def test_full_size_config(gpu_lib):
    """16 rows x 2^16 coefficients (1024 ring columns), 256 witnesses in [0, 256)."""
    from morpheus_gb300.ajtai import AjtaiKey
    key = np.array([0xC0FFEE, 1, 2, 3, 4, 5, 6, 7], np.uint32)
    n_ring, B = 1024, 256
    z8 = np.random.default_rng(3).integers(0, 256, size=(B, n_ring * 64), dtype=np.uint8)
    k = AjtaiKey(key, 0, 16, n_ring)
    out = k.commit_u8_batched(z8)
    assert out.shape == (B, 16, 64) and (out < Q).all()
    pick = [0, 255]
    assert np.array_equal(out[pick], O.ajtai_commit_u8_batch(key, z8[pick], row_lo=0, nrows=16))
