"""Basefold on the GPU against the CPU oracle: reference-ABI kernels, commit, open_ext2."""
import ctypes

import numpy as np
import pytest

import oracle as O

P = O.P
pytestmark = pytest.mark.gpu


def rnd(seed, *shape):
    return np.random.default_rng(seed).integers(0, P, size=shape, dtype=np.uint64)


_KEEP = []


@pytest.fixture(autouse=True)
def _release_buffers():
    """Buffers made by dev() live until the test ends: a temporary passed as
    dev(x).ptr would otherwise be freed before the kernel that reads it runs."""
    yield
    _KEEP.clear()


def dev(arr):
    from morpheus_gb300.memory import DeviceBuffer
    buf = DeviceBuffer.from_numpy(np.ascontiguousarray(arr, dtype=np.uint64).reshape(-1))
    _KEEP.append(buf)
    return buf


def canon(x):
    x = np.asarray(x, dtype=np.uint64)
    return np.where(x >= np.uint64(P), x - np.uint64(P), x)


# ---------------------------------------------------------------- Poseidon2 / Merkle
def test_poseidon2_batch_matches_reference_code(gpu_lib, golden):
    cases = golden["poseidon2_ref"]["cases"]
    inp = np.array([c[0] for c in cases], np.uint64)
    out = dev(np.zeros_like(inp))
    assert gpu_lib.poseidon2_hash_batch_ffi(dev(inp).ptr, out.ptr, len(cases)) == 0
    got = canon(out.to_numpy().reshape(-1, 8))
    assert got.tolist() == [c[1] for c in cases]


@pytest.mark.parametrize("leaves", [1, 2, 8, 1024, 4096, 1 << 15, 1 << 17])
def test_merkle_tree_gl_and_ext2(gpu_lib, leaves):
    from morpheus_gb300.memory import DeviceBuffer
    cw = rnd(leaves, 2 * leaves)
    tree = DeviceBuffer((2 * leaves - 1) * 4)
    assert gpu_lib.poseidon2_merkle_tree_gl_ffi(dev(cw).ptr, tree.ptr, leaves) == 0
    assert np.array_equal(canon(tree.to_numpy()), O.merkle_tree_gl(cw))
    cw2 = rnd(leaves + 1, 4 * leaves)
    assert gpu_lib.poseidon2_merkle_tree_ext2_ffi(dev(cw2).ptr, tree.ptr, leaves) == 0
    assert np.array_equal(canon(tree.to_numpy()), O.merkle_tree_ext2(cw2))


@pytest.mark.parametrize("parents", [1 << 13, 1 << 14, 1 << 15, 1 << 16])
def test_merkle_layer_every_form(gpu_lib, parents):
    """One layer at the sizes where the launch switches form (cooperative, pair, one thread)."""
    from morpheus_gb300.memory import DeviceBuffer
    layer = rnd(parents, 2 * parents, 4)
    out = DeviceBuffer(4 * parents)
    assert gpu_lib.poseidon2_merkle_layer_ffi(dev(layer).ptr, out.ptr, parents) == 0
    got = canon(out.to_numpy().reshape(parents, 4))
    for j in (0, 1, parents // 2 + 3, parents - 1):
        r = np.zeros(4, np.uint64)
        O.lib().or_poseidon2_compress(layer[2 * j].copy(), layer[2 * j + 1].copy(), r)
        assert np.array_equal(got[j], r), j


def test_merkle_layer_and_compress(gpu_lib):
    from morpheus_gb300.memory import DeviceBuffer
    layer = rnd(3, 64, 4)
    out = DeviceBuffer(32 * 4)
    assert gpu_lib.poseidon2_merkle_layer_ffi(dev(layer).ptr, out.ptr, 32) == 0
    exp = []
    for j in range(32):
        r = np.zeros(4, np.uint64)
        O.lib().or_poseidon2_compress(layer[2 * j].copy(), layer[2 * j + 1].copy(), r)
        exp.append(r)
    assert np.array_equal(canon(out.to_numpy().reshape(32, 4)), np.array(exp))
    l, r = rnd(4, 16, 4), rnd(5, 16, 4)
    assert gpu_lib.poseidon2_compress_batch_ffi(dev(l).ptr, dev(r).ptr, out.ptr, 16) == 0
    got = canon(out.to_numpy().reshape(32, 4)[:16])
    for j in range(16):
        e = np.zeros(4, np.uint64)
        O.lib().or_poseidon2_compress(l[j].copy(), r[j].copy(), e)
        assert np.array_equal(got[j], e)


# ---------------------------------------------------------------- eq, interp, encode
@pytest.mark.parametrize("n", [0, 1, 5, 12, 13, 16])
def test_eq_tables(gpu_lib, n):
    from morpheus_gb300.memory import DeviceBuffer
    r = rnd(n + 50, max(n, 1), 2)[:n]
    a, b = DeviceBuffer(2 << n), DeviceBuffer(2 << n)
    res = ctypes.c_void_p()
    assert gpu_lib.ext2_eq_dp_all_ffi(dev(r).ptr if n else dev(np.zeros(2, np.uint64)).ptr, a.ptr, b.ptr, n,
                                      ctypes.byref(res)) == 0
    which = a if res.value == a.ptr.value else b
    assert res.value == (b.ptr.value if n % 2 else a.ptr.value)
    got = canon(which.to_numpy().reshape(-1, 2))
    assert np.array_equal(got, O.eq_table_ext2(r.reshape(-1, 2)) if n else np.array([[1, 0]], np.uint64))
    rb = rnd(n + 60, max(n, 1))[:n]
    a1, b1 = DeviceBuffer(1 << n), DeviceBuffer(1 << n)
    assert gpu_lib.eq_dp_all_ffi(dev(rb).ptr if n else dev(np.zeros(1, np.uint64)).ptr, a1.ptr, b1.ptr, n,
                                 ctypes.byref(res)) == 0
    w = a1 if res.value == a1.ptr.value else b1
    exp = np.zeros(1 << n, np.uint64)
    O.lib().or_eq_table_base(rb if n else np.zeros(1, np.uint64), n, exp)
    assert np.array_equal(canon(w.to_numpy()), exp)


@pytest.mark.parametrize("n,lr", [(1, 1), (4, 1), (9, 2), (14, 1), (11, 3)])
def test_bhc_interpolate_and_encode(gpu_lib, n, lr):
    from morpheus_gb300.memory import DeviceBuffer
    ev = rnd(n, 1 << n)
    co_ref, bh_ref = O.bhc_interpolate(ev)
    co, bh = DeviceBuffer(1 << n), DeviceBuffer(1 << n)
    assert gpu_lib.basefold_bhc_interpolate_ffi(dev(ev).ptr, co.ptr, bh.ptr, n) == 0
    assert np.array_equal(canon(co.to_numpy()), co_ref)
    assert np.array_equal(canon(bh.to_numpy()), bh_ref)
    cw = DeviceBuffer(1 << (n + lr))
    assert gpu_lib.basefold_encode_ffi(dev(co_ref).ptr, cw.ptr, n, lr) == 0
    assert np.array_equal(canon(cw.to_numpy()), O.basefold_encode(co_ref, lr))


def test_bit_reverse(gpu_lib):
    x = dev(np.arange(16, dtype=np.uint64))
    assert gpu_lib.basefold_bit_reverse_gl_ffi(x.ptr, 4) == 0
    assert x.to_numpy().tolist() == [int(format(i, "04b")[::-1], 2) for i in range(16)]
    y = dev(np.arange(32, dtype=np.uint64))
    assert gpu_lib.basefold_bit_reverse_ext2_ffi(y.ptr, 4) == 0
    got = y.to_numpy().reshape(16, 2)
    assert got[:, 0].tolist() == [2 * int(format(i, "04b")[::-1], 2) for i in range(16)]


# ---------------------------------------------------------------- folds & sumcheck helpers
def emul(a, b):
    return ((a[0] * b[0] + 7 * a[1] * b[1]) % P, (a[0] * b[1] + a[1] * b[0]) % P)


def test_fold_kernels(gpu_lib):
    from morpheus_gb300.memory import DeviceBuffer
    pairs = 300
    tab = rnd(1, pairs, 2)
    cwb = rnd(2, 2 * pairs)
    cwe = rnd(3, 2 * pairs, 2)
    ch = [int(x) for x in rnd(4, 2)]
    out = DeviceBuffer(2 * pairs)
    assert gpu_lib.basefold_fold_gl_ffi(dev(cwb).ptr, dev(tab).ptr, ch[0], out.ptr, pairs) == 0
    g = canon(out.to_numpy()[:pairs])
    for i in range(0, pairs, 7):
        v0, v1, x0, w = int(cwb[2 * i]), int(cwb[2 * i + 1]), int(tab[i, 0]), int(tab[i, 1])
        assert int(g[i]) == (v0 + (ch[0] - x0) * (v1 - v0) * w) % P
    assert gpu_lib.basefold_fold_mixed_ffi(dev(cwb).ptr, dev(tab).ptr, ch[0], ch[1], out.ptr, pairs) == 0
    g = canon(out.to_numpy().reshape(pairs, 2))
    for i in range(0, pairs, 7):
        v0, v1, x0, w = int(cwb[2 * i]), int(cwb[2 * i + 1]), int(tab[i, 0]), int(tab[i, 1])
        f = emul(((ch[0] - x0) % P, ch[1]), (((v1 - v0) * w) % P, 0))
        assert (int(g[i, 0]), int(g[i, 1])) == ((v0 + f[0]) % P, f[1])
    assert gpu_lib.basefold_fold_ext2_ffi(dev(cwe).ptr, dev(tab).ptr, ch[0], ch[1], out.ptr, pairs) == 0
    g = canon(out.to_numpy().reshape(pairs, 2))
    for i in range(0, pairs, 7):
        v0, v1 = [int(x) for x in cwe[2 * i]], [int(x) for x in cwe[2 * i + 1]]
        x0, w = int(tab[i, 0]), int(tab[i, 1])
        dw = (((v1[0] - v0[0]) * w) % P, ((v1[1] - v0[1]) * w) % P)
        f = emul(((ch[0] - x0) % P, ch[1]), dw)
        assert (int(g[i, 0]), int(g[i, 1])) == ((v0[0] + f[0]) % P, (v0[1] + f[1]) % P)


def test_sumcheck_product_eval_interp_dot(gpu_lib):
    from morpheus_gb300.memory import DeviceBuffer
    pairs = 1000
    blocks = 4
    eq = rnd(10, 2 * pairs, 2)
    bh = rnd(11, 2 * pairs)
    bhe = rnd(12, 2 * pairs, 2)
    p0, p1, p2 = DeviceBuffer(2 * blocks), DeviceBuffer(2 * blocks), DeviceBuffer(2 * blocks)

    def red(buf):
        v = buf.to_numpy().reshape(blocks, 2).astype(object).sum(axis=0) % P
        return (int(v[0]), int(v[1]))

    def expect(e, b):
        c0 = c1 = c2 = (0, 0)
        for i in range(pairs):
            ee, eo = e[2 * i], e[2 * i + 1]
            be, bo = b[2 * i], b[2 * i + 1]
            add = lambda x, y: ((x[0] + y[0]) % P, (x[1] + y[1]) % P)
            c0 = add(c0, emul(ee, be))
            c1 = add(c1, add(emul(ee, bo), emul(eo, be)))
            c2 = add(c2, emul(eo, bo))
        return c0, c1, c2

    E = [(int(a), int(b)) for a, b in eq]
    Bb = [(int(a), 0) for a in bh]
    Be = [(int(a), int(b)) for a, b in bhe]
    assert gpu_lib.basefold_sumcheck_product_mixed_ffi(dev(eq).ptr, dev(bh).ptr, p0.ptr, p1.ptr, p2.ptr, pairs, blocks) == 0
    assert (red(p0), red(p1), red(p2)) == expect(E, Bb)
    assert gpu_lib.basefold_sumcheck_product_ext2_ffi(dev(eq).ptr, dev(bhe).ptr, p0.ptr, p1.ptr, p2.ptr, pairs, blocks) == 0
    assert (red(p0), red(p1), red(p2)) == expect(E, Be)
    # fused eval + interp + product == eval, interp, product separately
    ch = [int(x) for x in rnd(13, 2)]
    eo, bo = DeviceBuffer(2 * pairs * 2), DeviceBuffer(2 * pairs * 2)
    q = pairs // 2
    assert gpu_lib.fused_sumcheck_round_ext2_ffi(dev(eq).ptr, dev(bhe).ptr, ch[0], ch[1], eo.ptr, bo.ptr, p0.ptr,
                                                 p1.ptr, p2.ptr, q, blocks) == 0
    fused = (red(p0), red(p1), red(p2))
    e_ev, b_ev = DeviceBuffer(2 * pairs), DeviceBuffer(2 * pairs)
    assert gpu_lib.basefold_sumcheck_eval_ext2_ffi(dev(eq).ptr, ch[0], ch[1], e_ev.ptr, pairs) == 0
    assert gpu_lib.basefold_sumcheck_eval_ext2_ffi(dev(bhe).ptr, ch[0], ch[1], b_ev.ptr, pairs) == 0
    assert gpu_lib.basefold_sumcheck_interp_ext2_ffi(e_ev.ptr, q) == 0
    assert gpu_lib.basefold_sumcheck_interp_ext2_ffi(b_ev.ptr, q) == 0
    assert np.array_equal(canon(e_ev.to_numpy()), canon(eo.to_numpy()[:2 * pairs]))
    assert gpu_lib.basefold_sumcheck_product_ext2_ffi(e_ev.ptr, b_ev.ptr, p0.ptr, p1.ptr, p2.ptr, q, blocks) == 0
    assert (red(p0), red(p1), red(p2)) == fused
    # dot products
    dpp = DeviceBuffer(2 * blocks)
    assert gpu_lib.basefold_dot_product_mixed_ffi(dev(bh).ptr, dev(eq).ptr, dpp.ptr, 2 * pairs, blocks) == 0
    exp = [0, 0]
    for i in range(2 * pairs):
        exp[0] = (exp[0] + int(bh[i]) * int(eq[i, 0])) % P
        exp[1] = (exp[1] + int(bh[i]) * int(eq[i, 1])) % P
    assert red(dpp) == tuple(exp)


# ---------------------------------------------------------------- commit / open drivers
@pytest.mark.parametrize("n,lr", [(1, 1), (2, 1), (5, 2), (8, 1), (10, 3), (13, 1)])
def test_commit_matches_oracle(gpu_lib, n, lr):
    from morpheus_gb300.basefold import BasefoldCommitment
    ev = rnd(200 + n, 1 << n)
    ref = O.basefold_commit(ev, lr)
    c = BasefoldCommitment.commit(ev, n, lr)
    assert np.array_equal(c.root, ref["root"])
    assert np.array_equal(canon(c.codeword()), ref["codeword"])
    assert np.array_equal(canon(c.tree()), ref["tree"])


def test_table_matches_oracle(gpu_lib):
    from morpheus_gb300.basefold import BasefoldTable
    t = BasefoldTable.generate(9, 3, 9, 42)
    ent, off = O.basefold_table(9, 3, 9, 42)
    assert np.array_equal(t.entries(), ent)
    assert np.array_equal(t.level_offsets(), off)


# n = 16 folds 2^15- and 2^14-leaf rounds (the pair-form launches) and 2^16-parent layers
@pytest.mark.parametrize("n,lr,q,table_nv", [(2, 1, 3, 2), (4, 1, 4, 6), (6, 3, 10, 9), (9, 1, 34, 9), (12, 1, 34, 14),
                                             (11, 2, 7, 11), (16, 1, 34, 16)])
def test_open_ext2_matches_oracle(gpu_lib, n, lr, q, table_nv):
    from morpheus_gb300.basefold import BasefoldCommitment, BasefoldTable
    from morpheus_gb300.sumcheck import Transcript
    ev = rnd(300 + n, 1 << n)
    pt = rnd(301 + n, n, 2)
    ref_c = O.basefold_commit(ev, lr)
    table_h = O.basefold_table(table_nv, lr, table_nv, 42)
    t = O.Transcript(b"bf-open")
    t.append_ext2(b"", [5, 6])
    t.append_u64(b"", 3)
    ref = O.basefold_open_ext2(ref_c, pt, table_h, t, q)

    c = BasefoldCommitment.commit(ev, n, lr)
    tab = BasefoldTable.generate(table_nv, lr, table_nv, 42)
    tg = Transcript(b"bf-open")
    tg.append_ext2(b"", [5, 6])
    tg.append_u64(b"", 3)
    proof = c.open_ext2(pt, tab, tg, q)
    assert np.array_equal(proof, ref)
    tv = O.Transcript(b"bf-open")
    tv.append_ext2(b"", [5, 6])
    tv.append_u64(b"", 3)
    assert O.basefold_verify_ext2(c.root, n, lr, pt, proof, q, table_h, tv)
    # transcripts end in the same state
    assert np.array_equal(tg.challenge_ext2(b"x"), t.challenge_ext2(b"x"))


def test_full_size_commit_open_verify(gpu_lib):
    """The bench workload: 2^22 evaluations, rate 1/2, 34 queries, table seed 42."""
    from morpheus_gb300.basefold import BasefoldCommitment, BasefoldTable, split_proof
    from morpheus_gb300.sumcheck import Transcript
    n, lr, q = 22, 1, 34
    ev = rnd(22, 1 << n)
    pt = rnd(23, n, 2)
    tab = BasefoldTable.generate(n, lr, n, 42)
    c = BasefoldCommitment.commit(ev, n, lr)
    t = Transcript(b"bf-open")
    proof = c.open_ext2(pt, tab, t, q)
    sp = split_proof(proof, n, lr, q)
    assert np.array_equal(sp["eval"], O.ml_eval_ext2(ev, pt))
    table_h = (tab.entries(), tab.level_offsets())
    tv = O.Transcript(b"bf-open")
    assert O.basefold_verify_ext2(c.root, n, lr, pt, proof, q, table_h, tv)
    bad = proof.copy()
    bad[len(bad) // 3] ^= np.uint64(1)
    assert not O.basefold_verify_ext2(c.root, n, lr, pt, bad, q, table_h, O.Transcript(b"bf-open"))
    # the committed codeword is 2 copies of one block (rate 1/2), and its root matches an
    # independent oracle tree over a slice: hash of leaf 0 and of leaf 2^(n-1) agree
    tree = c.tree()
    assert np.array_equal(tree[:4], tree[4 * (1 << (n - 1)): 4 * (1 << (n - 1)) + 4])
