"""Ajtai commitment on the GPU against the reference's own CPU code (golden vectors) and the oracle."""
import numpy as np
import pytest

import oracle as O

Q = O.Q_AGL
pytestmark = pytest.mark.gpu


@pytest.fixture(params=[1, 2, 3, 4], ids=["circulant", "toeplitz", "toeplitz-pair", "hankel-pair"])
def form(request, gpu_lib):
    """Runs the test once with each tensor-core form of the batched commitment."""
    from morpheus_gb300.ajtai import batch_form
    with batch_form(request.param):
        yield request.param


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


def test_batched_matches_reference(gpu_lib, form, golden):
    from morpheus_gb300.ajtai import AjtaiKey
    g = golden["ajtai_commit_u8_ref"]
    k = AjtaiKey(g["key"], 0, g["rows"], g["N"])
    out = k.commit_u8_batched(np.array(g["z"], np.uint8).reshape(1, -1))
    assert [int(x) for x in out.reshape(-1)] == g["out"]


# shapes cover one and several K chunks per tile, tiles whose chunks span many CTAs of the
# persistent schedule (1 row x 1024 ring columns: 38 slots), two witness tiles (B > 256) and K padding
@pytest.mark.parametrize("n_ring,B,row_lo,rows", [(16, 3, 0, 16), (40, 5, 0, 16), (8, 130, 3, 2), (33, 1, 40, 2),
                                                  (1024, 2, 0, 1), (64, 300, 5, 1)])
def test_batched_vs_oracle(gpu_lib, form, n_ring, B, row_lo, rows):
    from morpheus_gb300.ajtai import AjtaiKey
    key = np.array([9, 8, 7, 6, 5, 4, 3, 2], np.uint32)
    z8 = np.random.default_rng(n_ring + B).integers(0, 256, size=(B, n_ring * 64), dtype=np.uint8)
    k = AjtaiKey(key, row_lo, rows, n_ring)
    out = k.commit_u8_batched(z8)
    pick = sorted({0, B - 1, B // 2})
    ref = O.ajtai_commit_u8_batch(key, z8[pick], row_lo=row_lo, nrows=rows)
    assert np.array_equal(out[pick], ref)


def test_batched_extremes_and_batch_invariance(gpu_lib, form):
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


def test_batched_unaligned_witness_pointer(gpu_lib, form):
    """A witness array that is not 8-byte aligned takes the one-coefficient-per-thread prep."""
    import ctypes
    from morpheus_gb300.ajtai import AjtaiKey
    from morpheus_gb300.memory import DeviceBuffer
    key = np.array([3, 1, 4, 1, 5, 9, 2, 6], np.uint32)
    n_ring, B = 16, 3
    z8 = np.random.default_rng(5).integers(0, 256, size=(B, n_ring * 64), dtype=np.uint8)
    raw = np.zeros(B * n_ring * 64 + 8, np.uint8)
    raw[1:1 + z8.size] = z8.reshape(-1)
    buf = DeviceBuffer.from_numpy(raw)

    class _At:  # a device address one byte into the buffer
        ptr = ctypes.c_void_p(buf.ptr.value + 1)

    k = AjtaiKey(key, 0, 2, n_ring)
    out = k.commit_u8_batched((_At(), B))
    assert np.array_equal(out, k.commit_u8_batched(z8))
    assert np.array_equal(out[[0, 2]], O.ajtai_commit_u8_batch(key, z8[[0, 2]], row_lo=0, nrows=2))


def test_batched_equals_wide_rows(gpu_lib, form):
    from morpheus_gb300 import ajtai
    key = np.array([11, 22, 33, 44, 55, 66, 77, 88], np.uint32)
    n_ring = 16
    z8 = np.random.default_rng(2).integers(0, 256, size=(2, n_ring * 64), dtype=np.uint8)
    out = ajtai.AjtaiKey(key, 0, 42, n_ring).commit_u8_batched(z8)
    for b in range(2):
        assert np.array_equal(out[b], ajtai.commit_wide(key, z8[b].astype(np.uint64)))


def test_full_size_config(gpu_lib, form):
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


def _dev(a):
    from morpheus_gb300.memory import DeviceBuffer
    return DeviceBuffer.from_numpy(np.ascontiguousarray(a))


def _bits_to_coeffs(words, neg_words=None):
    """u64 bitmasks -> full-width coefficients (1, q - 1 for -1, 0)"""
    out = np.zeros((len(words), 64), np.uint64)
    for j, w in enumerate(words):
        for l in range(64):
            v = (int(w) >> l) & 1
            if neg_words is not None:
                v -= (int(neg_words[j]) >> l) & 1
            out[j, l] = v % Q
    return out.reshape(-1)


def test_dense_batched_matches_reference_and_oracle(gpu_lib, golden):
    from morpheus_gb300 import _native as N
    L = N.lib()
    g = golden["ajtai_commit_binary_ref"]
    key = np.array(g["key"], np.uint32)
    z = np.array(g["z_bits"], np.uint64)
    d_key, d_z, d_out = _dev(key), _dev(z), _dev(np.zeros(42 * 64, np.uint64))
    assert L.ajtai_commit_dense_batched_ffi(d_key.ptr, d_z.ptr, len(z), 1, 64, d_out.ptr) == 0
    assert [int(x) for x in d_out.to_numpy()] == g["out"]
    # a batch of 5 witnesses against a column window
    rng = np.random.default_rng(4)
    n, B, off = 37, 5, 9
    zb = rng.integers(0, 1 << 63, size=(B, n), dtype=np.uint64) | (rng.integers(0, 2, size=(B, n), dtype=np.uint64) << np.uint64(63))
    d_zb, d_ob = _dev(zb), _dev(np.zeros(B * 42 * 64, np.uint64))
    assert L.ajtai_commit_dense_batched_at_ffi(d_key.ptr, d_zb.ptr, n, B, 256, off, d_ob.ptr) == 0
    got = d_ob.to_numpy().reshape(B, 42, 64)
    for b in range(B):
        assert np.array_equal(got[b], O.ajtai_commit_wide(key, _bits_to_coeffs(zb[b]), off, 0, 42))
    assert L.ajtai_commit_dense_batched_ffi(d_key.ptr, d_zb.ptr, n, 17, 64, d_ob.ptr) == -2
    assert L.ajtai_commit_dense_batched_ffi(d_key.ptr, d_zb.ptr, n, 2, 100, d_ob.ptr) == -3


def test_ternary_and_sparse_vs_oracle(gpu_lib):
    from morpheus_gb300 import _native as N
    L = N.lib()
    rng = np.random.default_rng(8)
    key = np.array([9, 9, 8, 8, 7, 7, 6, 6], np.uint32)
    n = 21
    # the 13 ternary chunks of a split witness, committed together (ajtai.cuh:1262-1370)
    pos = rng.integers(0, 1 << 63, size=(13, n), dtype=np.uint64)
    neg = rng.integers(0, 1 << 63, size=(13, n), dtype=np.uint64) & ~pos
    d_key, d_out = _dev(key), _dev(np.zeros(13 * 42 * 64, np.uint64))
    d_pos, d_neg = _dev(pos), _dev(neg)
    assert L.ajtai_commit_ternary_ffi(d_key.ptr, d_pos.ptr, d_neg.ptr, n, 1024, d_out.ptr) == 0
    got = d_out.to_numpy().reshape(13, 42, 64)
    for i in (0, 6, 12):
        assert np.array_equal(got[i], O.ajtai_commit_wide(key, _bits_to_coeffs(pos[i], neg[i]), 0, 0, 42))
    # the same against a materialized matrix (ajtai_premat.cuh)
    d_M = _dev(np.zeros(n * 42 * 64, np.uint64))
    assert L.ajtai_materialize_m_ffi(d_key.ptr, d_M.ptr, n) == 0
    M = d_M.to_numpy().reshape(n, 42, 64)
    assert np.array_equal(M[5, 3], O.ajtai_ring_elem(key, 3, 5)) and np.array_equal(M[20, 41], O.ajtai_ring_elem(key, 41, 20))
    d_out2 = _dev(np.zeros(13 * 42 * 64, np.uint64))
    assert L.ajtai_commit_ternary_premat_ffi(d_M.ptr, d_pos.ptr, d_neg.ptr, n, 256, d_out2.ptr) == 0
    assert np.array_equal(d_out2.to_numpy(), d_out.to_numpy())
    assert L.ajtai_commit_ternary_premat_ffi(d_M.ptr, d_pos.ptr, d_neg.ptr, n, 100, d_out2.ptr) == -3
    # sparse positions (ascending with gaps, one repeated index counted twice) across > 1 chunk
    cols = 700
    p = np.sort(rng.choice(cols * 64, size=300, replace=False)).astype(np.uint64)
    p = np.concatenate([p[:150], p[149:150], p[150:]])
    coeff = np.zeros(cols * 64, np.uint64)
    for x in p:
        coeff[int(x)] += 1
    d_p = _dev(p)
    d_out = _dev(np.zeros(42 * 64, np.uint64))
    assert L.ajtai_commit_sparse_ffi(d_key.ptr, d_p.ptr, len(p), 64, d_out.ptr) == 0
    assert np.array_equal(d_out.to_numpy().reshape(42, 64), O.ajtai_commit_wide(key, coeff, 0, 0, 42))
    assert L.ajtai_commit_sparse_ffi(d_key.ptr, d_p.ptr, 0, 64, d_out.ptr) == 0 and not d_out.to_numpy().any()


def test_gemm_bounded_waits_time_out_and_the_context_recovers(gpu_lib, form):
    """The tensor-core GEMM's mbarrier waits are bounded.  In the starved test mode the producer
    issues no operand loads, so the MMA and epilogue waits can only run out: the call must return
    -1 with the wait's code in gb_last_error(), and the next normal call on the same context must
    be bit-exact (TMEM released, no copy left in flight)."""
    import re
    from morpheus_gb300 import ajtai, _native as N
    L = N.lib()
    key = np.array([3, 1, 4, 1, 5, 9, 2, 6], np.uint32)
    k = ajtai.AjtaiKey(key, 0, 16, 64)
    z8 = np.random.default_rng(31).integers(0, 256, size=(5, 64 * 64), dtype=np.uint8)
    want = O.ajtai_commit_u8_batch(key, z8, 0, 16)
    old = L.gb_ajtai_test_starve(1)
    try:
        with pytest.raises(N.NativeError) as exc:
            k.commit_u8_batched(z8)
        msg = L.gb_last_error().decode()
        m = re.search(r"pipeline wait timed out \(code (\d+)\)", msg)
        assert m and 1 <= int(m.group(1)) <= 11, msg
        assert "gb_ajtai_commit_u8_batched" in str(exc.value)
    finally:
        assert L.gb_ajtai_test_starve(old) == 1
    for _ in range(2):
        assert np.array_equal(k.commit_u8_batched(z8), want)


@pytest.mark.parametrize("B", [1, 4, 5, 6, 104, 105, 300])
def test_batch_forms_agree(gpu_lib, B):
    """The four tensor-core forms and the automatic choice (witness-circulant up to 104 witnesses,
    the Hankel-window pair GEMM above) give the same commitments, on either side of the threshold
    and over several witness tiles."""
    from morpheus_gb300.ajtai import AjtaiKey, batch_form
    key = np.array([2, 7, 1, 8, 2, 8, 1, 8], np.uint32)
    n_ring = 48
    z8 = np.random.default_rng(B).integers(0, 256, size=(B, n_ring * 64), dtype=np.uint8)
    k = AjtaiKey(key, 1, 16, n_ring)
    outs = []
    for f in (0, 1, 2, 3, 4):
        with batch_form(f):
            outs.append(k.commit_u8_batched(z8))
    assert all(np.array_equal(outs[0], o) for o in outs[1:])
    pick = sorted({0, B - 1})
    assert np.array_equal(outs[0][pick], O.ajtai_commit_u8_batch(key, z8[pick], row_lo=1, nrows=16))


def test_batch_form_rejects_out_of_range(gpu_lib):
    from morpheus_gb300 import _native as N
    L = N.lib()
    assert L.gb_ajtai_set_batch_form(5) == -2 and L.gb_ajtai_set_batch_form(-1) == -2
    assert L.gb_ajtai_set_batch_form(0) == 0


def test_key_expansion_is_built_on_first_large_batch(gpu_lib):
    """A key that only ever commits small batches holds its 16 MB of digit planes, not the 1.07 GB
    Toeplitz expansion; the first batch in the key-Toeplitz form builds the expansion, and both
    forms stay bit-exact around it."""
    import ctypes
    from morpheus_gb300 import _native as N
    from morpheus_gb300.ajtai import AjtaiKey, batch_form
    L = N.lib()

    def free_bytes():
        f, t = ctypes.c_size_t(), ctypes.c_size_t()
        assert L.cuda_mem_get_info(ctypes.byref(f), ctypes.byref(t)) == 0
        return f.value

    key = np.array([4, 4, 2, 2, 1, 1, 0, 7], np.uint32)
    z8 = np.random.default_rng(77).integers(0, 256, size=(3, 1024 * 64), dtype=np.uint8)
    want = O.ajtai_commit_u8_batch(key, z8[:1], 0, 16)
    f0 = free_bytes()
    k = AjtaiKey(key, 0, 16, 1024)
    assert np.array_equal(k.commit_u8_batched(z8[:1]), want)
    assert f0 - free_bytes() < (512 << 20)
    with batch_form(2):
        out = k.commit_u8_batched(z8)
    assert f0 - free_bytes() > (1 << 30)
    assert np.array_equal(out[:1], want)
    with batch_form(1):
        assert np.array_equal(k.commit_u8_batched(z8), out)
