"""Ajtai commitment over almost-Goldilocks, mirroring almost-goldilocks-cuda-rs/src/ajtai.rs.

``commit_wide`` keeps the crate's name and arguments (ajtai.rs:299-344): a witness
of full-width coefficients against the column window starting at ``col_offset``,
returning KAPPA = 42 rows of 64 canonical coefficients.  ``AjtaiKey`` is the
batched tensor-core path for witnesses with coefficients in [0, 256).
"""
import ctypes

import numpy as np

from . import _native as N
from .memory import DeviceBuffer

KAPPA = 42
RING_DIM = 64
Q = 0xFFFFFFFEFFFFFFE1


def commit_wide(seed, z_wide, col_offset=0, chunk=None):
    """seed: 8 u32; z_wide: N*64 canonical coefficients.  Returns [42][64] canonical."""
    z = np.ascontiguousarray(np.asarray(z_wide, dtype=np.uint64).reshape(-1))
    if z.size == 0 or z.size % RING_DIM:
        raise ValueError("z_wide length must be a nonzero multiple of 64")
    n_ring = z.size // RING_DIM
    d_z = DeviceBuffer.from_numpy(z)
    d_key = DeviceBuffer.from_numpy(np.asarray(seed, dtype=np.uint32))
    d_out = DeviceBuffer(KAPPA * RING_DIM)
    N.check(N.lib().ajtai_commit_wide_ffi(d_key.ptr, d_z.ptr, n_ring, col_offset, chunk or 256, d_out.ptr),
            "ajtai_commit_wide_ffi")
    return d_out.to_numpy().reshape(KAPPA, RING_DIM)


class batch_form:
    """Context manager: the calling thread's form of AjtaiKey.commit_u8_batched (0 by batch size,
    1 witness-circulant GEMM, 2 key-Toeplitz GEMM, 3 key-Toeplitz GEMM on CTA pairs, 4 the pair
    GEMM on the key's Hankel windows; gb_ajtai_set_batch_form).  Results never depend on it."""

    def __init__(self, form):
        self.form = form

    def __enter__(self):
        self._old = N.lib().gb_ajtai_set_batch_form(self.form)
        N.check(self._old if self._old < 0 else 0, "gb_ajtai_set_batch_form")
        return self

    def __exit__(self, *a):
        N.lib().gb_ajtai_set_batch_form(self._old)


class AjtaiKey:
    """Rows [row_lo, row_lo + rows) of the matrix over n_ring columns, with the GEMM operands each
    built once: the digit planes (16 MB for 16 rows x 1024 columns) at creation, their Hankel
    windows (252 MB) and their Toeplitz expansion (1.07 GB) by the first batch whose form reads
    them."""

    def __init__(self, seed, row_lo, rows, n_ring):
        self.rows, self.n_ring = rows, n_ring
        self.handle = ctypes.c_void_p()
        s = np.ascontiguousarray(np.asarray(seed, dtype=np.uint32))
        N.check(N.lib().gb_ajtai_key_create(s.ctypes.data, row_lo, rows, n_ring, ctypes.byref(self.handle)),
                "gb_ajtai_key_create")

    def commit_u8_batched(self, z8):
        """z8: [B][n_ring*64] uint8 (host array or DeviceBuffer with B given as tuple (buf, B)).
        Returns [B][rows][64] canonical coefficients."""
        if isinstance(z8, tuple):
            dz, B = z8
        else:
            arr = np.ascontiguousarray(np.asarray(z8, dtype=np.uint8))
            B = arr.shape[0]
            assert arr.shape[1] == self.n_ring * RING_DIM
            dz = DeviceBuffer.from_numpy(arr.reshape(-1))
        out = DeviceBuffer(B * self.rows * RING_DIM)
        N.check(N.lib().gb_ajtai_commit_u8_batched(self.handle, dz.ptr, B, out.ptr), "gb_ajtai_commit_u8_batched")
        return out.to_numpy().reshape(B, self.rows, RING_DIM)

    def __del__(self):
        try:
            if self.handle:
                N.lib().gb_ajtai_key_destroy(self.handle)
                self.handle = None
        except Exception:
            pass
