"""The fold tree's other sumcheck provers through the C ABI (almost-goldilocks-cuda-rs ffi.rs:141-160,
:319-400) against big-integer restatements of almost_sumcheck_prover.cuh:360-700 and the sparse
boolean check of almost wrapper.cu:2652-2980, with per-block partials grouped as the reference's
grid-stride loops group them (block b takes the items with (i mod blocks*256) // 256 == b)."""
import ctypes

import numpy as np
import pytest

import oracle as O

pytestmark = pytest.mark.gpu
Q = O.Q_AGL
BLOCK = 256
_KEEP = []


@pytest.fixture(autouse=True)
def _release_buffers():
    yield
    _KEEP.clear()


def dev(arr, dt=np.uint64):
    from morpheus_gb300.memory import DeviceBuffer
    buf = DeviceBuffer.from_numpy(np.ascontiguousarray(arr, dtype=dt).reshape(-1))
    _KEEP.append(buf)
    return buf


def mul(a, b):
    return ((a[0] * b[0] + 3 * a[1] * b[1]) % Q, (a[0] * b[1] + a[1] * b[0]) % Q)


def add(a, b):
    return ((a[0] + b[0]) % Q, (a[1] + b[1]) % Q)


def sub(a, b):
    return ((a[0] - b[0]) % Q, (a[1] - b[1]) % Q)


def rnd_e2(rng, n):
    return [tuple(int(x) for x in rng.integers(0, Q, 2, dtype=np.uint64)) for _ in range(n)]


def bit(words, i):
    return (int(words[i // 64]) >> (i % 64)) & 1


def blk(i, blocks):
    return (i % (blocks * BLOCK)) // BLOCK


def test_build_fu_and_wide_to_ternary(gpu_lib):
    from morpheus_gb300 import _native as N
    L = N.lib()
    rng = np.random.default_rng(1)
    n, leaves, uniques = 300, 7, 3
    words = (n + 63) // 64
    pos = rng.integers(0, 2**63, size=(leaves, words), dtype=np.uint64)
    neg = rng.integers(0, 2**63, size=(leaves, words), dtype=np.uint64) & ~pos
    alphas = rnd_e2(rng, leaves)
    leaf_u = [0, 2, 1, 0, 2, 2, 1]
    order = sorted(range(leaves), key=lambda l: leaf_u[l])
    offs = [0] + [sum(1 for l in leaf_u if l <= u) for u in range(uniques)]
    for tern in (False, True):
        d_fu = dev(np.zeros(uniques * n * 2))
        args = (dev(np.array(alphas, np.uint64)).ptr, dev(order, np.int32).ptr, dev(offs, np.int32).ptr, d_fu.ptr, n,
                uniques, words)
        rc = L.aext2_build_fu_ternary_ffi(dev(pos).ptr, dev(neg).ptr, *args) if tern else \
            L.aext2_build_fu_ffi(dev(pos).ptr, *args)
        assert rc == 0
        got = d_fu.to_numpy().reshape(uniques, n, 2)
        for u in range(uniques):
            for x in (0, 1, 63, 64, 200, n - 1):
                want = (0, 0)
                for l in range(leaves):
                    if leaf_u[l] != u:
                        continue
                    if bit(pos[l], x):
                        want = add(want, alphas[l])
                    if tern and bit(neg[l], x):
                        want = sub(want, alphas[l])
                assert tuple(int(v) for v in got[u, x]) == want
    # device split into k planes, with the error flag
    z = rng.integers(-1000, 1001, size=(50, 64)).astype(np.int16)
    for k, bad in ((10, False), (9, True)):
        d_p, d_n, d_e = dev(np.zeros(k * 50)), dev(np.zeros(k * 50)), dev(np.zeros(1, np.int32), np.int32)
        assert L.aext2_wide_to_ternary_ffi(dev(z, np.int16).ptr, d_p.ptr, d_n.ptr, d_e.ptr, 50, k) == 0
        L.cuda_sync_mine()
        wp, wn = O.ajtai_split_witness(z)
        assert np.array_equal(d_p.to_numpy().reshape(k, 50), wp[:k]) and np.array_equal(d_n.to_numpy().reshape(k, 50), wn[:k])
        assert int(d_e.to_numpy()[0]) == int(bad)
    assert L.aext2_wide_to_ternary_ffi(dev(z, np.int16).ptr, d_p.ptr, d_n.ptr, d_e.ptr, 50, 17) == -1


def test_eq_suffix_factored_and_shared_messages(gpu_lib):
    from morpheus_gb300 import _native as N
    L = N.lib()
    rng = np.random.default_rng(2)
    log_n, uniques, blocks = 6, 2, 2
    n = 1 << log_n
    stride = 2 * n
    R = [rnd_e2(rng, log_n) for _ in range(uniques)]
    d_r = dev(np.array([c for r in R for e in r for c in e], np.uint64))
    d_eqs = dev(np.zeros(uniques * stride))
    assert L.aext2_eq_suffix_dp_ffi(d_r.ptr, d_eqs.ptr, log_n, uniques, stride) == 0
    eqs = d_eqs.to_numpy().reshape(uniques, n, 2)

    def eqsuf(u, t, y):  # prod_{i >= t} eq1(R_i, bit i-t of y)
        v = (1, 0)
        for i in range(t, log_n):
            b = (y >> (i - t)) & 1
            v = mul(v, R[u][i] if b else sub((1, 0), R[u][i]))
        return v
    for u in range(uniques):
        for t in range(1, log_n + 1):
            size = 1 << (log_n - t)
            for y in range(size):
                assert tuple(int(x) for x in eqs[u, size - 1 + y]) == eqsuf(u, t, y)
    # factored message on round t: eqsuf_{t+1} (offset 2^(n-t-1) - 1, half = 2^(n-t-1))
    F = [rnd_e2(rng, n) for _ in range(uniques)]
    d_f = dev(np.array(F, np.uint64))
    t = 2
    half = 1 << (log_n - t - 1)
    d_part = dev(np.zeros(blocks * uniques * 4))
    assert L.aext2_sharedeq_factored_msg_ffi(d_eqs.ptr, d_f.ptr, d_part.ptr, half - 1, stride, 2 * n, half, uniques,
                                             blocks) == 0
    got = d_part.to_numpy().reshape(blocks, uniques, 2, 2)
    for u in range(uniques):
        want = [[(0, 0), (0, 0)] for _ in range(blocks)]
        for y in range(half):
            e = eqsuf(u, t + 1, y)
            b = blk(y, blocks)
            want[b][0] = add(want[b][0], mul(e, F[u][2 * y]))
            want[b][1] = add(want[b][1], mul(e, F[u][2 * y + 1]))
        assert [[tuple(int(x) for x in got[b, u, c]) for c in range(2)] for b in range(blocks)] == want
    # unfactored message and the single fold
    leaves, half = 4, 300
    orig = 2 * half
    l2u = [1, 0, 1, 0]
    EQ = [rnd_e2(rng, orig) for _ in range(2)]
    FF = [rnd_e2(rng, orig) for _ in range(leaves)]
    d_part = dev(np.zeros(blocks * leaves * 6))
    assert L.aext2_sharedeq_msg_ffi(dev(np.array(EQ, np.uint64)).ptr, dev(np.array(FF, np.uint64)).ptr,
                                    dev(l2u, np.int32).ptr, d_part.ptr, orig, half, leaves, blocks) == 0
    got = d_part.to_numpy().reshape(blocks, leaves, 3, 2)
    for leaf in range(leaves):
        want = [[(0, 0)] * 3 for _ in range(blocks)]
        E, Fv = EQ[l2u[leaf]], FF[leaf]
        for y in range(half):
            b = blk(y, blocks)
            e2 = sub(add(E[2 * y + 1], E[2 * y + 1]), E[2 * y])
            f2 = sub(add(Fv[2 * y + 1], Fv[2 * y + 1]), Fv[2 * y])
            terms = [mul(E[2 * y], Fv[2 * y]), mul(E[2 * y + 1], Fv[2 * y + 1]), mul(e2, f2)]
            want[b] = [add(want[b][c], terms[c]) for c in range(3)]
        assert [[tuple(int(x) for x in got[b, leaf, c]) for c in range(3)] for b in range(blocks)] == want
    ch = rnd_e2(rng, 1)[0]
    d_in, d_out = dev(np.array(FF, np.uint64)), dev(np.zeros(leaves * orig * 2))
    assert L.aext2_fold_single_ffi(d_in.ptr, d_out.ptr, ch[0], ch[1], orig, half, leaves) == 0
    out = d_out.to_numpy().reshape(leaves, orig, 2)
    for leaf in range(leaves):
        for y in (0, 7, half - 1):
            a, b2 = FF[leaf][2 * y], FF[leaf][2 * y + 1]
            assert tuple(int(x) for x in out[leaf, y]) == add(a, mul(ch, sub(b2, a)))


def bool_round_ref(terms, w, eq):
    """one round of the sparse boolean check restated: terms = list of sorted (idx, val) lists"""
    msg = [(0, 0)] * 4
    pairs = []
    for t, entries in enumerate(terms):
        pos_map = dict(entries)
        seen = set()
        for idx, _ in entries:
            rest = idx >> 1
            if rest in seen:
                continue
            seen.add(rest)
            v0, v1 = pos_map.get(2 * rest, (0, 0)), pos_map.get(2 * rest + 1, (0, 0))
            q0, q1 = eq[2 * rest], eq[2 * rest + 1]
            for c in range(4):
                v = add(v0, mul((c, 0), sub(v1, v0)))
                q = add(q0, mul((c, 0), sub(q1, q0)))
                msg[c] = add(msg[c], mul(mul(w[t], mul(v, sub(v, (1, 0)))), q))
            pairs.append((t, rest, v0, v1))
    return msg, pairs


def test_sparse_boolean_check_rounds(gpu_lib):
    from morpheus_gb300 import _native as N
    L = N.lib()
    rng = np.random.default_rng(4)
    n_terms, log_n, grid_x = 5, 9, 2
    terms = []
    for t in range(n_terms):
        k = int(rng.integers(1, 60)) if t != 2 else 1
        idx = sorted(int(x) for x in rng.choice(1 << log_n, size=k, replace=False))
        terms.append([(i, (1, 0)) for i in idx])
    w = rnd_e2(rng, n_terms)
    n = sum(len(t) for t in terms)
    d_idx = dev(np.array([i for t in terms for i, _ in t], np.uint32), np.uint32)
    d_val = dev(np.zeros(2 * n))
    assert L.agl_bool_init_val_ffi(d_val.ptr, n) == 0
    assert (d_val.to_numpy().reshape(n, 2) == [1, 0]).all()
    off = [0]
    for t in terms:
        off.append(off[-1] + len(t))
    d_off = dev(np.array(off, np.uint32), np.uint32)
    for rd in range(log_n):
        size = 1 << (log_n - rd)
        eq = rnd_e2(rng, size)
        want_msg, pairs = bool_round_ref(terms, w, eq)
        d_flags, d_gid = dev(np.zeros(n, np.uint32), np.uint32), dev(np.zeros(n, np.uint32), np.uint32)
        d_part = dev(np.zeros(grid_x * n_terms * 8))
        d_scr = dev(np.zeros(4 * ((n + 255) // 256) + 8, np.uint32), np.uint32)
        h_msg = np.zeros(8, np.uint64)
        h_total = ctypes.c_uint32()
        assert L.agl_bool_round_msg_ffi(d_idx.ptr, d_val.ptr, d_off.ptr, dev(np.array(w, np.uint64)).ptr,
                                        dev(np.array(eq, np.uint64)).ptr, n_terms, n, d_flags.ptr, d_gid.ptr,
                                        d_part.ptr, grid_x, d_scr.ptr, d_scr.len, h_msg.ctypes.data,
                                        ctypes.byref(h_total)) == 0
        assert [tuple(int(x) for x in h_msg[2 * c:2 * c + 2]) for c in range(4)] == want_msg
        assert h_total.value == len(pairs)
        ch = rnd_e2(rng, 1)[0]
        d_oi, d_ov = dev(np.zeros(n, np.uint32), np.uint32), dev(np.zeros(2 * n))
        d_no = dev(np.zeros(n_terms + 1, np.uint32), np.uint32)
        assert L.agl_bool_fold_ffi(d_idx.ptr, d_val.ptr, d_flags.ptr, d_gid.ptr, d_off.ptr, n_terms, n, ch[0], ch[1],
                                   h_total.value, grid_x, d_oi.ptr, d_ov.ptr, d_no.ptr) == 0
        # restated fold: each pair -> (rest, v0 + ch (v1 - v0)), terms in order
        new_terms = [[] for _ in range(n_terms)]
        for t, rest, v0, v1 in pairs:
            new_terms[t].append((rest, add(v0, mul(ch, sub(v1, v0)))))
        n2 = h_total.value
        gi, gv = d_oi.to_numpy()[:n2], d_ov.to_numpy().reshape(-1, 2)[:n2]
        assert [(int(i), (int(v[0]), int(v[1]))) for i, v in zip(gi, gv)] == [e for t in new_terms for e in t]
        no = [int(x) for x in d_no.to_numpy()]
        want_off = [0]
        for t in new_terms:
            want_off.append(want_off[-1] + len(t))
        assert no == want_off
        terms, n, d_idx, d_val, d_off = new_terms, n2, d_oi, d_ov, d_no
    d_fin = dev(np.zeros(2 * n_terms))
    assert L.agl_bool_finish_ffi(d_idx.ptr, d_val.ptr, d_off.ptr, n_terms, n, d_fin.ptr) == 0
    fin = d_fin.to_numpy().reshape(n_terms, 2)
    for t in range(n_terms):
        want = terms[t][0][1] if terms[t] and terms[t][0][0] == 0 else (0, 0)
        assert tuple(int(x) for x in fin[t]) == want
