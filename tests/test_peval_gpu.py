"""Partial evaluation, bit permutation and the fused permute + partial evaluation through the C ABI
(goldilocks-cuda-rs partial_eval_gl_ffi, partial_eval_ext2_from_gl_ffi, bit_permute_gl_ffi,
fused_permute_partial_eval_ffi and the almost-goldilocks forms) against the oracle's restatement,
on the reference's own test inputs (goldilocks-cuda-rs/src/partial_eval.rs:524-720) and on einsum
shapes with the reference's range permutations (zk-torch-3/src/bin/bench_permute_partial.rs)."""
import ctypes

import numpy as np
import pytest

import oracle as O

pytestmark = pytest.mark.gpu
P = O.P
QA = O.Q_AGL
MOD = {"gl": P, "agl": QA}


def ref_evals(n, mod):
    return np.array([((i + 1) * 0xDEADBEEFCAFEBABE % 2**64) % mod for i in range(n)], np.uint64)


def ref_r(m, mod, ext):
    a = [((i + 1) * 12345678901234567 % 2**64) % mod for i in range(m)]
    if not ext:
        return np.array(a, np.uint64)
    b = [((i + 1) * 98765432109876543 % 2**64) % mod for i in range(m)]
    return np.array(list(zip(a, b)), np.uint64)


@pytest.mark.parametrize("field", ["gl", "agl"])
@pytest.mark.parametrize("log_n", [4, 8, 12, 16])
def test_partial_eval_reference_cases(gpu_lib, field, log_n):
    from morpheus_gb300 import partial_eval as PE
    mod = MOD[field]
    ev = ref_evals(1 << log_n, mod)
    for m in sorted({1, log_n // 2, log_n}):
        r = ref_r(m, mod, False)
        assert np.array_equal(PE.partial_eval_base(ev, r, field), O.partial_eval_base(ev, r, field))
        re = ref_r(m, mod, True)
        assert np.array_equal(PE.partial_eval_ext2(ev, re, field), O.partial_eval_ext2(ev, re, field))


@pytest.mark.parametrize("field", ["gl", "agl"])
@pytest.mark.parametrize("log_n,m", [(1, 1), (5, 3), (9, 4), (10, 9), (13, 5), (22, 9), (22, 13)])
def test_partial_eval_random(gpu_lib, field, log_n, m):
    from morpheus_gb300 import partial_eval as PE
    mod = MOD[field]
    rng = np.random.default_rng(log_n * 31 + m)
    ev = rng.integers(0, 2**64 - 1, size=1 << log_n, dtype=np.uint64)  # non-canonical inputs too
    r = rng.integers(0, mod, size=m, dtype=np.uint64)
    re = rng.integers(0, mod, size=(m, 2), dtype=np.uint64)
    if field == "agl":
        ev = ev % np.uint64(mod)
    assert np.array_equal(PE.partial_eval_base(ev, r, field), O.partial_eval_base(ev, r, field))
    assert np.array_equal(PE.partial_eval_ext2(ev, re, field), O.partial_eval_ext2(ev, re, field))


def test_partial_eval_reference_edge_cases(gpu_lib):
    """partial_eval.rs:650-720: m = 0 is the identity, f(0,0) = evals[0], f(1,1) = evals[3], and an
    Ext2 r with c1 = 0 gives the base result."""
    from morpheus_gb300 import partial_eval as PE
    ev = np.array([1, 2, 3, 4], np.uint64)
    assert PE.partial_eval_base(ev, []).tolist() == [1, 2, 3, 4]
    assert PE.partial_eval_base(ev, [0, 0]).tolist() == [1]
    assert PE.partial_eval_base(ev, [1, 1]).tolist() == [4]
    assert PE.partial_eval_ext2(ev, np.zeros((0, 2), np.uint64)).tolist() == [[1, 0], [2, 0], [3, 0], [4, 0]]
    e = PE.partial_eval_ext2(ev, [[7, 0]])
    assert e[:, 0].tolist() == PE.partial_eval_base(ev, [7]).tolist() and e[:, 1].tolist() == [0, 0]
    assert PE.partial_eval_ext2(ev, [[0, 0], [0, 0]]).tolist() == [[1, 0]]
    # m <= 0 leaves the data untouched (the reference returns before launching)
    from morpheus_gb300 import _native as N
    from morpheus_gb300.memory import DeviceBuffer
    d = DeviceBuffer.from_numpy(ev)
    assert N.lib().partial_eval_gl_ffi(d.ptr, d.ptr, 2, 0) == 0
    assert d.to_numpy().tolist() == [1, 2, 3, 4]


@pytest.mark.parametrize("field", ["gl", "agl"])
@pytest.mark.parametrize("n_bits", [0, 1, 3, 5, 7, 12, 20])
def test_bit_permute(gpu_lib, field, n_bits):
    from morpheus_gb300 import partial_eval as PE
    from morpheus_gb300.memory import DeviceBuffer
    rng = np.random.default_rng(n_bits)
    x = rng.integers(0, 2**64 - 1, size=1 << n_bits, dtype=np.uint64)
    for trial in range(3):
        perm = list(rng.permutation(n_bits)) if trial else list(range(n_bits))[::-1]
        inv = [0] * n_bits
        for old, new in enumerate(perm):
            inv[new] = old
        d_in, d_out = DeviceBuffer.from_numpy(x), DeviceBuffer(1 << n_bits)
        PE.bit_permute(d_in, d_out, [int(p) for p in perm], field)
        assert np.array_equal(d_out.to_numpy(), O.bit_permute(x, inv))


def test_bit_permute_rejects_non_permutation(gpu_lib):
    from morpheus_gb300 import _native as N
    from morpheus_gb300.memory import DeviceBuffer
    d = DeviceBuffer(16)
    bad = DeviceBuffer.from_numpy(np.array([0, 0, 1, 2], np.int32))
    assert N.lib().bit_permute_gl_ffi(d.ptr, d.ptr, bad.ptr, 4, 16) == -2
    ok = DeviceBuffer.from_numpy(np.array([0, 1, 2, 3], np.int32))
    assert N.lib().bit_permute_gl_ffi(d.ptr, d.ptr, ok.ptr, 4, 15) == -2  # total != 2^n_bits


def eq_table(ch, field):
    if field == "gl":
        return O.eq_table_ext2(ch).reshape(-1, 2)
    q, w = QA, 3
    out = [(1, 0)]
    for c0, c1 in [(int(a), int(b)) for a, b in ch]:
        omr = ((1 - c0) % q, (-c1) % q)
        nxt = [None] * (2 * len(out))
        for j, (a0, a1) in enumerate(out):
            nxt[j] = ((a0 * omr[0] + w * a1 * omr[1]) % q, (a0 * omr[1] + a1 * omr[0]) % q)
            nxt[j + len(out)] = ((a0 * c0 + w * a1 * c1) % q, (a0 * c1 + a1 * c0) % q)
        out = nxt
    return np.array(out, np.uint64)


def swap_halves(lo_bits, hi_bits):
    """The einsum A-input range permutation (bench_permute_partial.rs): [(j, j + i), (0, j)]."""
    return [(lo_bits, lo_bits + hi_bits), (0, lo_bits)]


@pytest.mark.parametrize("field", ["gl", "agl"])
@pytest.mark.parametrize("n,m,ranges", [
    (12, 6, swap_halves(6, 6)),          # square transpose, m = the former high half
    (16, 4, swap_halves(12, 4)),         # many outputs, short sums
    (16, 12, swap_halves(4, 12)),        # few outputs, long sums (split-sum path)
    (20, 18, swap_halves(2, 18)),        # 4 outputs
    (18, 7, [(0, 3), (10, 18), (3, 10)]),
    (14, 14, swap_halves(7, 7)),         # full evaluation: one output
    (3, 2, [(2, 3), (0, 2)]),            # fewer than 5 index bits
    (10, 0, swap_halves(5, 5)),
])
def test_fused_permute_partial_eval(gpu_lib, field, n, m, ranges):
    from morpheus_gb300 import partial_eval as PE
    mod = MOD[field]
    rng = np.random.default_rng(n * 7 + m)
    ev = rng.integers(0, mod, size=1 << n, dtype=np.uint64)
    ch = rng.integers(0, mod, size=(m, 2), dtype=np.uint64)
    got = PE.fused_permute_partial_eval(ev, ch, ranges, n, field)
    if m == 0:
        assert np.array_equal(got[:, 0], ev) and not got[:, 1].any()
        return
    half = n // 2
    lo, hi = PE.build_split_luts(n, ranges, half)
    want = O.fused_permute_peval(ev, n, m, half, eq_table(ch, field), lo, hi, field)
    assert np.array_equal(got, want)
    # the same as a bit permutation followed by a partial evaluation
    perm = PE.perm_from_ranges(n, ranges)
    inv = [0] * n
    for old, new in enumerate(perm):
        inv[new] = old
    assert np.array_equal(got, O.partial_eval_ext2(O.bit_permute(ev, inv), ch, field))


def test_fused_output_prefix_and_invalid(gpu_lib):
    """output_size below 2^(n-m) writes only that prefix; larger or zero is rejected."""
    from morpheus_gb300 import _native as N
    from morpheus_gb300 import partial_eval as PE
    from morpheus_gb300.memory import DeviceBuffer
    n, m = 12, 5
    rng = np.random.default_rng(3)
    ev = rng.integers(0, P, size=1 << n, dtype=np.uint64)
    ch = rng.integers(0, P, size=(m, 2), dtype=np.uint64)
    ranges = swap_halves(5, 7)
    full = PE.fused_permute_partial_eval(ev, ch, ranges, n)
    lo, hi = PE.build_split_luts(n, ranges, n // 2)
    d_ev, d_lo, d_hi = DeviceBuffer.from_numpy(ev), DeviceBuffer.from_numpy(lo), DeviceBuffer.from_numpy(hi)
    d_eq = DeviceBuffer.from_numpy(eq_table(ch, "gl").reshape(-1))
    out = DeviceBuffer.from_numpy(np.full(2 << (n - m), 7, np.uint64))
    L = N.lib()
    assert L.fused_permute_partial_eval_ffi(d_ev.ptr, out.ptr, d_eq.ptr, d_lo.ptr, d_hi.ptr, n, m, n // 2, 100, 0) == 0
    L.cuda_sync_mine()
    got = out.to_numpy().reshape(-1, 2)
    assert np.array_equal(got[:100], full[:100]) and (got[100:] == 7).all()
    for outs in (0, (1 << (n - m)) + 1):
        assert L.fused_permute_partial_eval_ffi(d_ev.ptr, out.ptr, d_eq.ptr, d_lo.ptr, d_hi.ptr, n, m, n // 2,
                                                outs, 0) == -2
