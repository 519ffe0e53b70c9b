"""The CPU oracle against the reference's golden vectors and its own code (CPU only)."""
import os

import numpy as np
import pytest

import oracle as O

P = O.P
Q = O.Q_AGL


def test_gl_ops_match_reference_device_code(golden):
    L = O.lib()
    for a, b, add, sub, mul in golden["gl_ops_ref"]["cases"]:
        assert L.or_gl_add(a, b) == add
        assert L.or_gl_sub(a, b) == sub
        assert L.or_gl_mul(a, b) == mul


def test_gl_mul_against_bigint():
    rng = np.random.default_rng(7)
    L = O.lib()
    for a, b in rng.integers(0, 2**64, size=(500, 2), dtype=np.uint64):
        assert L.or_gl_mul(int(a), int(b)) == (int(a) * int(b)) % P
    assert L.or_gl_inv(0) == 0
    for a in [1, 2, 7, P - 1, 123456789]:
        assert (L.or_gl_inv(a) * a) % P == 1


def test_ext2_mul_matches_reference(golden):
    for a, b, out in golden["ext2_mul_ref"]["cases"]:
        r = np.zeros(2, np.uint64)
        O.lib().or_ext2_mul(np.array(a, np.uint64), np.array(b, np.uint64), r)
        assert [int(x) for x in r] == out


def test_poseidon2_matches_reference_code(golden):
    for inp, out in golden["poseidon2_ref"]["cases"]:
        assert [int(x) for x in O.poseidon2_permute(np.array(inp, np.uint64))] == out


def test_poseidon2_reference_kat_is_not_the_reference_permutation(golden):
    # The reference's standalone test prints a Plonky3 vector that its own permutation
    # does not produce; the oracle follows the reference code (pinned above).
    kat = golden["poseidon2_plonky3_kat"]
    got = [int(x) for x in O.poseidon2_permute(np.array(kat["input"], np.uint64))]
    assert got != kat["expected"]
    assert got == golden["poseidon2_ref"]["cases"][0][1]


def test_almost_goldilocks_golden(golden):
    L = O.lib()
    for a, b, exp in golden["agl_add_golden"]["cases"]:
        assert L.or_agl_add(a, b) == exp
    for a, b, exp in golden["agl_mul_golden"]["cases"]:
        assert L.or_agl_mul(a, b) == exp
    for a, b, exp in golden["aext2_mul_golden"]["cases"]:
        r = np.zeros(2, np.uint64)
        L.or_aext2_mul(np.array(a, np.uint64), np.array(b, np.uint64), r)
        assert [int(x) for x in r] == exp


def test_chacha8_and_prg_match_reference(golden):
    for key, ctr, nonce, out in golden["chacha8_ref"]["cases"]:
        r = np.zeros(16, np.uint32)
        O.lib().or_chacha8_block(np.array(key, np.uint32), ctr, np.array(nonce, np.uint32), r)
        assert [int(x) for x in r] == out
    key = golden["ajtai_ring_elem_ref"]["key"]
    for row, j, out in golden["ajtai_ring_elem_ref"]["cases"]:
        assert [int(x) for x in O.ajtai_ring_elem(key, row, j)] == out


def test_ajtai_commit_matches_reference(golden):
    g = golden["ajtai_commit_wide_ref"]
    c = O.ajtai_commit_wide(g["key"], np.array(g["z"], np.uint64), col_offset=g["col_offset"], row_lo=0, nrows=g["rows"])
    assert [int(x) for x in c.reshape(-1)] == g["out"]
    g = golden["ajtai_commit_u8_ref"]
    z8 = np.array(g["z"], np.uint8).reshape(1, -1)
    c = O.ajtai_commit_u8_batch(g["key"], z8, row_lo=0, nrows=g["rows"])
    assert [int(x) for x in c.reshape(-1)] == g["out"]
    # binary witness = wide witness with 0/1 coefficients (ajtai_integration.rs:1198-1231 relation)
    g = golden["ajtai_commit_binary_ref"]
    bits = np.array([[(w >> l) & 1 for l in range(64)] for w in g["z_bits"]], np.uint64).reshape(-1)
    c = O.ajtai_commit_wide(g["key"], bits, 0, 0, 42)
    assert [int(x) for x in c.reshape(-1)] == g["out"]


def test_sumcheck_h70_both_modes(golden):
    g = golden["sumcheck_h70"]
    polys = np.array([g["p1"], g["p2"]], np.uint64)
    pr = O.sumcheck_prove_base(O.Transcript(g["labels"]["base"].encode()), polys)
    assert (int(pr["round_messages"][0][0]) + int(pr["round_messages"][0][1])) % P == g["sum"]
    pe = O.sumcheck_prove_ext2(O.Transcript(g["labels"]["ext2"].encode()), polys)
    m = pe["round_messages"]
    assert (int(m[0, 0, 0]) + int(m[0, 1, 0])) % P == g["sum"] and m[0, 0, 1] == 0
    assert O.sumcheck_verify_ext2(O.Transcript(g["labels"]["ext2"].encode()), 2, 2, [g["sum"], 0], m, pe["final_eval"])


@pytest.mark.parametrize("n,d", [(1, 1), (3, 2), (6, 3), (5, 4), (4, 8)])
def test_sumcheck_ext2_verifies_and_rejects_tamper(n, d):
    rng = np.random.default_rng(n * 10 + d)
    polys = rng.integers(0, P, size=(d, 1 << n), dtype=np.uint64)
    claim = 0
    prod = np.ones(1 << n, dtype=object)
    for i in range(d):
        prod = prod * polys[i].astype(object)
    claim = int(sum(prod) % P)
    pr = O.sumcheck_prove_ext2(O.Transcript(b"t"), polys)
    assert O.sumcheck_verify_ext2(O.Transcript(b"t"), n, d, [claim, 0], pr["round_messages"], pr["final_eval"])
    bad = pr["round_messages"].copy()
    bad[-1, -1, 0] = (int(bad[-1, -1, 0]) + 1) % P
    assert not O.sumcheck_verify_ext2(O.Transcript(b"t"), n, d, [claim, 0], bad, pr["final_eval"])


def test_eq_table_bit_order():
    rng = np.random.default_rng(3)
    r = rng.integers(0, P, size=(4, 2), dtype=np.uint64)
    eq = O.eq_table_ext2(r)

    def emul(a, b):
        return ((a[0] * b[0] + 7 * a[1] * b[1]) % P, (a[0] * b[1] + a[1] * b[0]) % P)

    for x in range(16):
        v = (1, 0)
        for i in range(4):
            ri = (int(r[i, 0]), int(r[i, 1]))
            term = ri if (x >> i) & 1 else ((1 - ri[0]) % P, (-ri[1]) % P)
            v = emul(v, term)
        assert (int(eq[x, 0]), int(eq[x, 1])) == v


def test_bhc_interpolation_reevaluates():
    # basefold.rs:3262-3297: sum of coeffs over subsets of x recovers evals[x]
    n = 5
    ev = np.random.default_rng(5).integers(0, P, size=1 << n, dtype=np.uint64)
    co, bh = O.bhc_interpolate(ev)
    for x in range(1 << n):
        s = sum(int(co[t]) for t in range(1 << n) if (x & t) == t) % P
        assert s == int(ev[x])
    rev = [int(ev[int(format(i, "05b")[::-1], 2)]) for i in range(1 << n)]
    assert [int(v) for v in bh] == rev


def test_encode_is_repeated_walsh_hadamard():
    n, lr = 4, 2
    co = np.random.default_rng(9).integers(0, P, size=1 << n, dtype=np.uint64)
    cw = O.basefold_encode(co, lr)
    wht = [sum(((-1) ** bin(c & s).count("1")) * int(co[s]) for s in range(1 << n)) % P for c in range(1 << n)]
    for j in range(1 << (n + lr)):
        o = int(format(j, f"0{n + lr}b")[::-1], 2)
        assert int(cw[j]) == wht[o >> lr]


def test_table_generation_deterministic():
    a = O.basefold_table(5, 1, 5, 42)
    b = O.basefold_table(5, 1, 5, 42)
    assert (a[0] == b[0]).all() and (a[1] == b[1]).all()
    assert (a[0][:, 1] != 0).all()
    assert list(a[1]) == [0, 32, 48, 56, 60]


@pytest.mark.parametrize("n,lr,q", [(2, 1, 3), (4, 1, 4), (6, 3, 10), (7, 1, 34)])
def test_basefold_open_verify_and_tamper(n, lr, q):
    rng = np.random.default_rng(100 + n)
    ev = rng.integers(0, P, size=1 << n, dtype=np.uint64)
    table = O.basefold_table(n + 2, lr, n + 2, 42)  # table for a larger max_num_vars, as the DAG does
    comm = O.basefold_commit(ev, lr)
    pt = rng.integers(0, P, size=(n, 2), dtype=np.uint64)
    t = O.Transcript(b"bf-open")
    t.append_u64(b"", 7)
    proof = O.basefold_open_ext2(comm, pt, table, t, q)
    # eval = multilinear extension at the point
    eq = O.eq_table_ext2(pt)
    e0 = sum(int(ev[i]) * int(eq[i, 0]) for i in range(1 << n)) % P
    e1 = sum(int(ev[i]) * int(eq[i, 1]) for i in range(1 << n)) % P
    assert (int(proof[0]), int(proof[1])) == (e0, e1)

    def ver(pf):
        tv = O.Transcript(b"bf-open")
        tv.append_u64(b"", 7)
        return O.basefold_verify_ext2(comm["root"], n, lr, pt, pf, q, table, tv)

    assert ver(proof)
    for pos in [0, 3, 2 + n * 6 + 1, len(proof) - 1, len(proof) // 2]:
        bad = proof.copy()
        bad[pos] = (int(bad[pos]) + 1) % P
        assert not ver(bad), pos


def test_agl_ext2_test_restatement_matches_pinned_oracle():
    """The big-integer Ext2 product the almost-Goldilocks GPU tests use equals the pinned oracle's."""
    import importlib.util, os
    spec = importlib.util.spec_from_file_location("tag", os.path.join(os.path.dirname(__file__), "test_agl_gpu.py"))
    tag = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(tag)
    rng = np.random.default_rng(0)
    for _ in range(20):
        a = [int(x) for x in rng.integers(0, O.Q_AGL, 2, dtype=np.uint64)]
        b = [int(x) for x in rng.integers(0, O.Q_AGL, 2, dtype=np.uint64)]
        assert list(tag.e2mul(a, b)) == [int(x) for x in O.aext2_mul(a, b)]


def test_monolith_oracle_matches_reference_kat(golden):
    """cpu_monolith.rs test vector: Monolith-12 of (0, 1, ..., 11)."""
    g = golden["monolith_kat"]
    assert [int(x) for x in O.monolith_permute(np.array(g["input"], np.uint64))] == g["expected"]


def test_monolith_oracle_tree_structure():
    """The oracle's trees: leaves are truncated permutations, parents compress their children."""
    cw = np.arange(100, 108, dtype=np.uint64)
    tree = O.monolith_tree_gl(cw).reshape(-1, 4)
    leaf0 = O.monolith_permute(np.array([100, 101] + [0] * 10, np.uint64))[:4]
    assert np.array_equal(tree[0], leaf0)
    parent = O.monolith_permute(np.concatenate([tree[0], tree[1], np.zeros(4, np.uint64)]))[:4]
    assert np.array_equal(tree[4], parent)
    assert tree.shape[0] == 7


def _bp_ref_point(a, b, n):
    return np.array([[((i + 1) * a) % O.P, ((i + 1) * b) % O.P] for i in range(n)], np.uint64)


@pytest.mark.parametrize("case", ["single", "same_point", "different_points"])
def test_batch_open_restatement_on_reference_tests(case):
    """batch_open_ext2 restated (basefold.rs:1202-1532) on the reference's own tests
    (basefold.rs:3908-4110): its restated verifier (:1931-2220) accepts, and rejects a wrong
    claim (the reference's tamper test, :4113-4170) and a flipped proof word."""
    n, lr, q = 4, 1, 4
    table = O.basefold_table(n, lr, n, 42)
    ea, eb = np.arange(1, 17, dtype=np.uint64), np.arange(100, 116, dtype=np.uint64)
    pa, pb = _bp_ref_point(111, 222, n), _bp_ref_point(333, 444, n)
    if case == "single":
        evals, points, pairs = [ea], [pa], [(0, 0)]
    elif case == "same_point":
        evals, points, pairs = [ea, eb], [pa], [(0, 0), (1, 0)]
    else:
        evals, points, pairs = [ea, eb], [pa, pb], [(0, 0), (1, 1)]
    comms = [O.basefold_commit(e, lr) for e in evals]
    claims = [(a, b, O.ml_eval_ext2(evals[a], points[b])) for a, b in pairs]
    proof = O.basefold_batch_open_ext2(comms, points, claims, table, O.Transcript(b"t"), q)
    assert proof.size == O.basefold_batch_proof_len(n, lr, q, len(claims))
    roots = [c["root"] for c in comms]
    assert O.basefold_batch_verify_ext2(roots, n, lr, points, claims, proof, q, table, O.Transcript(b"t"))
    bad = [(a, b, np.array([(int(v[0]) + 1) % O.P, int(v[1])], np.uint64)) for a, b, v in claims]
    assert not O.basefold_batch_verify_ext2(roots, n, lr, points, bad, proof, q, table, O.Transcript(b"t"))
    for k in (3, proof.size // 2, proof.size - 3):
        flip = proof.copy()
        flip[k] ^= np.uint64(1)
        assert not O.basefold_batch_verify_ext2(roots, n, lr, points, claims, flip, q, table, O.Transcript(b"t"))


def test_partial_eval_restatement_reference_cases():
    """The oracle's partial evaluation against the reference's CPU helpers restated in Python
    (goldilocks-cuda-rs/src/partial_eval.rs:449-520) on its own test inputs, and the reference's
    edge cases (:650-720)."""
    P = O.P
    for log_n in (4, 8):
        ev = [((i + 1) * 0xDEADBEEFCAFEBABE % 2**64) % P for i in range(1 << log_n)]
        for m in (1, log_n // 2, log_n):
            r = [((i + 1) * 12345678901234567 % 2**64) % P for i in range(m)]
            rc = [((i + 1) * 98765432109876543 % 2**64) % P for i in range(m)]
            d = list(ev)
            for ri in r:
                d = [(d[2 * j] + ri * (d[2 * j + 1] - d[2 * j])) % P for j in range(len(d) // 2)]
            assert O.partial_eval_base(np.array(ev, np.uint64), np.array(r, np.uint64)).tolist() == d
            e = [((ev[2 * j] + r[0] * (ev[2 * j + 1] - ev[2 * j])) % P, rc[0] * (ev[2 * j + 1] - ev[2 * j]) % P)
                 for j in range(len(ev) // 2)]
            for a, b in zip(r[1:], rc[1:]):
                nxt = []
                for j in range(len(e) // 2):
                    x, y = e[2 * j], e[2 * j + 1]
                    d0, d1 = (y[0] - x[0]) % P, (y[1] - x[1]) % P
                    nxt.append(((x[0] + a * d0 + 7 * b * d1) % P, (x[1] + a * d1 + b * d0) % P))
                e = nxt
            got = O.partial_eval_ext2(np.array(ev, np.uint64), np.array(list(zip(r, rc)), np.uint64))
            assert [tuple(int(v) for v in row) for row in got] == e
    ev = np.array([1, 2, 3, 4], np.uint64)
    assert O.partial_eval_base(ev, [0, 0]).tolist() == [1] and O.partial_eval_base(ev, [1, 1]).tolist() == [4]
    assert O.partial_eval_ext2(ev, [[7, 0]])[:, 0].tolist() == O.partial_eval_base(ev, [7]).tolist()


def test_fused_restatement_is_permute_then_partial_eval():
    rng = np.random.default_rng(5)
    n, m, half = 9, 4, 4
    ev = rng.integers(0, O.P, size=1 << n, dtype=np.uint64)
    ch = rng.integers(0, O.P, size=(m, 2), dtype=np.uint64)
    perm = list(rng.permutation(n))
    inv = [0] * n
    for old, new in enumerate(perm):
        inv[new] = old
    lo = np.array([sum(1 << inv[k] for k in range(half) if (x >> k) & 1) for x in range(1 << half)], np.uint32)
    hi = np.array([sum(1 << inv[half + k] for k in range(n - half) if (x >> k) & 1) for x in range(1 << (n - half))],
                  np.uint32)
    got = O.fused_permute_peval(ev, n, m, half, O.eq_table_ext2(ch), lo, hi)
    assert np.array_equal(got, O.partial_eval_ext2(O.bit_permute(ev, inv), ch))


def test_ext5_frobenius_constants():
    """The Ext5 Frobenius multipliers compiled into the library are the powers of 3^((p-1)/5),
    and 7, 3 are quadratic non-residues (their Frobenius multiplier is -1)."""
    import re
    src = open(os.path.join(os.path.dirname(__file__), "..", "morpheus_gb300", "csrc", "field_ops.cu")).read()
    m = re.search(r"c_frob_gl5\[5\] = \{([^}]*)\}", src)
    vals = [int(v.strip().rstrip("ull")) for v in m.group(1).split(",")]
    d = pow(3, (O.P - 1) // 5, O.P)
    assert vals == [pow(d, i, O.P) for i in range(5)]
    assert pow(7, (O.P - 1) // 2, O.P) == O.P - 1 and pow(3, (O.Q_AGL - 1) // 2, O.Q_AGL) == O.Q_AGL - 1


def test_poseidon2_zero_lane_sbox_constants():
    """The precomputed first-round S-boxes of zero lanes (leaf hashes) are rc_ext[0][i]^7 mod p."""
    import re
    src = open(os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "morpheus_gb300", "csrc",
                            "poseidon2.cuh")).read()
    rc = [int(x, 16) for x in re.findall(r"0x([0-9a-f]+)ull", src[src.index("#define GB_P2_RC_EXT"):
                                                                   src.index("#define GB_P2_RC_INT")])][:8]
    pre = [int(x, 16) for x in re.findall(r"0x([0-9a-f]+)ull", src[src.index("#define GB_P2_SBOX_RC0"):
                                                                    src.index("struct P2Const")])]
    assert pre == [pow(x % P, 7, P) for x in rc]
