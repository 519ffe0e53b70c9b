"""Device buffers over the library's own allocation/copy entry points.

Mirrors goldilocks-cuda-rs/src/memory.rs (DeviceBuffer<u64>): a typed,
caller-owned device allocation with from_slice / to_vec / read_slice.
"""
import ctypes

import numpy as np

from . import _native as N


class DeviceBuffer:
    """A device allocation of ``n`` elements of ``dtype`` (default u64)."""

    def __init__(self, n, dtype=np.uint64):
        self.dtype = np.dtype(dtype)
        self.len = int(n)
        self.nbytes = self.len * self.dtype.itemsize
        self.ptr = ctypes.c_void_p()
        if self.nbytes:
            N.check(N.lib().cuda_malloc(ctypes.byref(self.ptr), self.nbytes), "cuda_malloc")

    @classmethod
    def from_numpy(cls, arr):
        arr = np.ascontiguousarray(arr)
        buf = cls(arr.size, arr.dtype)
        if buf.nbytes:
            N.check(N.lib().cuda_memcpy_htod(buf.ptr, arr.ctypes.data, buf.nbytes), "cuda_memcpy_htod")
        return buf

    def to_numpy(self):
        out = np.empty(self.len, self.dtype)
        if self.nbytes:
            N.check(N.lib().cuda_memcpy_dtoh(out.ctypes.data, self.ptr, self.nbytes), "cuda_memcpy_dtoh")
        return out

    def read_slice(self, offset, count):
        out = np.empty(count, self.dtype)
        if count:
            src = ctypes.c_void_p(self.ptr.value + offset * self.dtype.itemsize)
            N.check(N.lib().cuda_memcpy_dtoh(out.ctypes.data, src, count * self.dtype.itemsize), "cuda_memcpy_dtoh")
        return out

    def at(self, offset):
        """Device address of element ``offset``."""
        return ctypes.c_void_p(self.ptr.value + offset * self.dtype.itemsize)

    def free(self):
        if self.ptr and self.ptr.value:
            N.lib().cuda_free(self.ptr)
            self.ptr = ctypes.c_void_p()

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass

    def __len__(self):
        return self.len


def synchronize():
    N.check(N.lib().cuda_device_synchronize(), "cuda_device_synchronize")
