"""ajtai_commit_wide_noalloc_ffi (static device scratch, no allocation) against
ajtai_commit_wide_ffi, called through the C ABI.  Collected after every other test file so
that it also runs after the rest of the suite has used the library."""
import numpy as np
import pytest

import oracle as O

pytestmark = pytest.mark.gpu
MAX_RING = 4096


def _commit(fn_name, key, z, n_ring, col_offset):
    from morpheus_gb300 import _native as N
    from morpheus_gb300.memory import DeviceBuffer
    d_key = DeviceBuffer.from_numpy(np.asarray(key, np.uint32))
    d_z = DeviceBuffer.from_numpy(np.ascontiguousarray(z, np.uint64))
    d_out = DeviceBuffer(42 * 64)
    try:
        N.check(getattr(N.lib(), fn_name)(d_key.ptr, d_z.ptr, n_ring, col_offset, 256, d_out.ptr), fn_name)
        return d_out.to_numpy().reshape(42, 64)
    finally:
        for b in (d_key, d_z, d_out):
            b.free()


def test_noalloc_matches_allocating_entry_two_calls_in_a_row(gpu_lib):
    rng = np.random.default_rng(77)
    cases = [(np.array([9, 8, 7, 6, 5, 4, 3, 2], np.uint32), 37, 5),
             (np.array([1, 1, 2, 3, 5, 8, 13, 21], np.uint32), 300, 1000)]
    outs = []
    for key, n_ring, off in cases:
        z = rng.integers(0, O.Q_AGL, size=n_ring * 64, dtype=np.uint64)
        got = _commit("ajtai_commit_wide_noalloc_ffi", key, z, n_ring, off)
        want = _commit("ajtai_commit_wide_ffi", key, z, n_ring, off)
        assert np.array_equal(got, want)
        outs.append(got)
    # the second call's smaller/larger chunk count leaves no trace of the first
    assert not np.array_equal(outs[0], outs[1])
    assert np.array_equal(_commit("ajtai_commit_wide_noalloc_ffi", cases[0][0],
                                  np.random.default_rng(77).integers(0, O.Q_AGL, size=37 * 64, dtype=np.uint64),
                                  37, 5), outs[0])


def test_noalloc_at_its_maximum_and_beyond(gpu_lib):
    from morpheus_gb300 import _native as N
    key = np.arange(8, dtype=np.uint32)
    z = np.random.default_rng(3).integers(0, 256, size=MAX_RING * 64, dtype=np.uint64)
    got = _commit("ajtai_commit_wide_noalloc_ffi", key, z, MAX_RING, 0)
    assert np.array_equal(got, _commit("ajtai_commit_wide_ffi", key, z, MAX_RING, 0))
    # one ring element more than the static scratch holds: rejected before any launch
    rc = N.lib().ajtai_commit_wide_noalloc_ffi(None, None, MAX_RING + 1, 0, 256, None)
    assert rc == -2
    assert b"exceeds" in N.lib().gb_last_error()


def test_noalloc_call_allocates_nothing(gpu_lib):
    """After a warm-up call, a call changes neither the free device memory nor the
    stream-ordered pool's high-water mark: no allocation happens on the request path."""
    import ctypes
    from morpheus_gb300 import _native as N
    from morpheus_gb300.memory import DeviceBuffer
    L = N.lib()
    key = np.array([4, 4, 2, 2, 1, 1, 0, 0], np.uint32)
    z = np.random.default_rng(11).integers(0, O.Q_AGL, size=MAX_RING * 64, dtype=np.uint64)
    d_key = DeviceBuffer.from_numpy(key)
    d_z = DeviceBuffer.from_numpy(z)
    d_out = DeviceBuffer(42 * 64)
    try:
        def call():
            N.check(L.ajtai_commit_wide_noalloc_ffi(d_key.ptr, d_z.ptr, MAX_RING, 0, 256, d_out.ptr),
                    "ajtai_commit_wide_noalloc_ffi")

        def free_bytes():
            f, t = ctypes.c_size_t(), ctypes.c_size_t()
            N.check(L.cuda_mem_get_info(ctypes.byref(f), ctypes.byref(t)), "cuda_mem_get_info")
            return f.value

        call()  # warm-up: may load the module and its static memory
        first = d_out.to_numpy()
        assert L.gb_pool_used_high(1) != ctypes.c_size_t(-1).value
        in_use = L.gb_pool_used_high(0)
        free0 = free_bytes()
        call()
        assert free_bytes() == free0
        assert L.gb_pool_used_high(0) == in_use
        assert np.array_equal(d_out.to_numpy(), first)
    finally:
        for b in (d_key, d_z, d_out):
            b.free()
