"""Partial evaluation and the fused permute + partial evaluation (einsum input preparation).

Mirrors goldilocks-cuda-rs/src/partial_eval.rs (partial_eval_gl, partial_eval_ext2,
fused_permute_partial_eval, build_split_luts) and almost-goldilocks-cuda-rs/src/partial_eval.rs
(partial_eval, partial_eval_ext2, fused_permute_partial_eval), plus GoldilocksOps::bit_permute
(goldilocks-cuda-rs/src/field.rs:186-224).  ``field="agl"`` selects the almost-Goldilocks forms.
Results are canonical numpy arrays (Ext2 values as [..., 2]).
"""
import ctypes

import numpy as np

from . import _native as N
from .memory import DeviceBuffer

_FFI = {
    "gl": ("partial_eval_gl_ffi", "partial_eval_ext2_from_gl_ffi", "fused_permute_partial_eval_ffi",
           "bit_permute_gl_ffi", "ext2_eq_dp_all_ffi"),
    "agl": ("agl_partial_eval_ffi", "agl_partial_eval_ext2_from_base_ffi", "agl_fused_permute_partial_eval_ffi",
            "agl_bit_permute_ffi", "aext2_eq_dp_all_ffi"),
}


def _log2_exact(n):
    if n <= 0 or n & (n - 1):
        raise ValueError("poly_evals length must be a positive power of two")
    return n.bit_length() - 1


def partial_eval_base(poly_evals, r, field="gl"):
    """f(r, x_{m+1..N}) for base-field r: 2^(N-m) base values (partial_eval_gl / partial_eval)."""
    ev = np.ascontiguousarray(np.asarray(poly_evals, np.uint64))
    r = np.ascontiguousarray(np.asarray(r, np.uint64).reshape(-1))
    log_n, m = _log2_exact(ev.size), r.size
    if m > log_n:
        raise ValueError(f"r length {m} exceeds log_n {log_n}")
    if m == 0:
        return ev.copy()
    d = DeviceBuffer.from_numpy(ev)
    dr = DeviceBuffer.from_numpy(r)
    N.check(getattr(N.lib(), _FFI[field][0])(d.ptr, dr.ptr, log_n, m), _FFI[field][0])
    N.check(N.lib().cuda_sync_mine(), "sync")
    return d.read_slice(0, 1 << (log_n - m))


def partial_eval_ext2(poly_evals, r, field="gl"):
    """f(r, x_{m+1..N}) for Ext2 r (base-field f): 2^(N-m) Ext2 values, shape [.., 2]."""
    ev = np.ascontiguousarray(np.asarray(poly_evals, np.uint64))
    r = np.ascontiguousarray(np.asarray(r, np.uint64).reshape(-1, 2))
    log_n, m = _log2_exact(ev.size), r.shape[0]
    if m > log_n:
        raise ValueError(f"r length {m} exceeds log_n {log_n}")
    if m == 0:
        return np.stack([ev, np.zeros_like(ev)], axis=1)
    d_in = DeviceBuffer.from_numpy(ev)
    dr = DeviceBuffer.from_numpy(r.reshape(-1))
    d_out = DeviceBuffer(2 * max(1, 1 << (log_n - 1)))
    N.check(getattr(N.lib(), _FFI[field][1])(d_in.ptr, d_out.ptr, dr.ptr, log_n, m), _FFI[field][1])
    N.check(N.lib().cuda_sync_mine(), "sync")
    return d_out.read_slice(0, 2 << (log_n - m)).reshape(-1, 2)


def perm_from_ranges(n, permute_ranges):
    """perm_map[old_var] = new position: the ranges' variables in order (partial_eval.rs:351-361)."""
    order = [v for start, end in permute_ranges for v in range(start, end)]
    if sorted(order) != list(range(n)):
        raise ValueError("permute_ranges must list every variable once")
    perm = [0] * n
    for new_pos, old_var in enumerate(order):
        perm[old_var] = new_pos
    return perm


def build_split_luts(n, permute_ranges, half):
    """(lo_lut, hi_lut): old index = lo_lut[new & (2^half - 1)] | hi_lut[new >> half]
    (goldilocks-cuda-rs/src/partial_eval.rs:345-401)."""
    perm = perm_from_ranges(n, permute_ranges)
    inv = [0] * n
    for old_var, new_pos in enumerate(perm):
        inv[new_pos] = old_var
    lo = np.zeros(1 << half, np.uint32)
    for k in range(half):
        lo[1 << k:2 << k] = lo[:1 << k] | np.uint32(1 << inv[k])
    hi = np.zeros(1 << (n - half), np.uint32)
    for k in range(n - half):
        hi[1 << k:2 << k] = hi[:1 << k] | np.uint32(1 << inv[half + k])
    return lo, hi


def eq_table_ext2_device(challenges, field="gl"):
    """The Ext2 eq table of the challenges on the device (ext2_eq_dp_all)."""
    ch = np.ascontiguousarray(np.asarray(challenges, np.uint64).reshape(-1))
    m = ch.size // 2
    d_r = DeviceBuffer.from_numpy(ch if ch.size else np.zeros(2, np.uint64))
    a, b = DeviceBuffer(2 << m), DeviceBuffer(2 << m)
    res = ctypes.c_void_p()
    N.check(getattr(N.lib(), _FFI[field][4])(d_r.ptr, a.ptr, b.ptr, m, ctypes.byref(res)), _FFI[field][4])
    return (a if res.value == a.ptr.value else b), (a, b, d_r)


def fused_permute_partial_eval(evals, challenges, permute_ranges, n, field="gl"):
    """out[j] = sum_b evals[perm(j 2^m + b)] eq(r, b): the partial evaluation at the m challenges
    of the evaluations with their variables reordered by permute_ranges, in one pass
    (partial_eval.rs:266-343).  Returns 2^(n-m) Ext2 values, shape [.., 2]."""
    ev = np.ascontiguousarray(np.asarray(evals, np.uint64))
    ch = np.asarray(challenges, np.uint64).reshape(-1, 2)
    m = ch.shape[0]
    assert ev.size == 1 << n and m <= n
    if m == 0:  # the reference returns the evaluations lifted, unpermuted (partial_eval.rs:280-283)
        return np.stack([ev, np.zeros_like(ev)], axis=1)
    half = n // 2
    lo, hi = build_split_luts(n, permute_ranges, half)
    d_ev = DeviceBuffer.from_numpy(ev)
    d_lo, d_hi = DeviceBuffer.from_numpy(lo), DeviceBuffer.from_numpy(hi)
    d_eq, keep = eq_table_ext2_device(ch, field)
    outs = 1 << (n - m)
    d_out = DeviceBuffer(2 * outs)
    smem = ((((1 << half) + (1 << (n - half))) * 4 + 7) & ~7) + 8 * 2 * 8
    N.check(getattr(N.lib(), _FFI[field][2])(d_ev.ptr, d_out.ptr, d_eq.ptr, d_lo.ptr, d_hi.ptr, n, m, half, outs,
                                             smem), _FFI[field][2])
    N.check(N.lib().cuda_sync_mine(), "sync")
    del keep
    return d_out.to_numpy().reshape(-1, 2)


def bit_permute(d_input, d_output, perm_map, field="gl"):
    """d_output[new] = d_input[old], perm_map[old_var] = new position (GoldilocksOps::bit_permute);
    both buffers on the device."""
    n_bits = len(perm_map)
    inv = np.zeros(max(n_bits, 1), np.int32)
    for old_var, new_pos in enumerate(perm_map):
        inv[new_pos] = old_var
    d_inv = DeviceBuffer.from_numpy(inv)
    N.check(getattr(N.lib(), _FFI[field][3])(d_input.ptr, d_output.ptr, d_inv.ptr, n_bits, 1 << n_bits),
            _FFI[field][3])
