"""CPU oracle for the prover field hot path -- TEST INFRASTRUCTURE ONLY.

This package is the checker: a plain-C restatement (oracle.c) of the reference's
CPU code, plus an optional host build of the reference's own Ajtai CPU reference
(_ref/).  Only tests/, ``__graft_entry__.smoke()`` and the CPU-baseline leg of
bench.py may import it.  The product package ``morpheus_gb300`` never does.

Parity pinning: the restatement is checked against the reference's golden
vectors (tests/golden/) and against the reference's own Ajtai code built from
its sources (oracle/_ref).
"""
import ctypes
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB = None
_REF = None

P = 0xFFFFFFFF00000001
Q_AGL = 0xFFFFFFFEFFFFFFE1

_u64p = np.ctypeslib.ndpointer(dtype=np.uint64, flags="C_CONTIGUOUS")
_u32p = np.ctypeslib.ndpointer(dtype=np.uint32, flags="C_CONTIGUOUS")
_u8p = np.ctypeslib.ndpointer(dtype=np.uint8, flags="C_CONTIGUOUS")
_i32p = np.ctypeslib.ndpointer(dtype=np.int32, flags="C_CONTIGUOUS")
_c = ctypes


def build(ref_root=None):
    """Compile liboracle.so, and _ref/ from the reference checkout at ref_root (default: the
    MORPHEUS_REFERENCE environment variable) when one is given and present."""
    subprocess.run(["make", "-s", "-C", _HERE, "liboracle.so"], check=True)
    if ref_root is None:
        ref_root = os.environ.get("MORPHEUS_REFERENCE")
    if ref_root and os.path.isdir(os.path.join(ref_root, "cuda_almost_goldilocks")):
        subprocess.run(["make", "-s", "-C", _HERE, "ref", f"REF={ref_root}"], check=True)


def lib():
    global _LIB
    if _LIB is None:
        path = os.path.join(_HERE, "liboracle.so")
        if not os.path.exists(path):
            build(ref_root="")
        L = ctypes.CDLL(path)
        u64, i32, sz = _c.c_uint64, _c.c_int, _c.c_size_t
        vp = _c.c_void_p
        for name, res, args in [
            ("or_set_threads", None, [i32]),
            ("or_get_threads", i32, []),
            ("or_gl_add", u64, [u64, u64]),
            ("or_gl_sub", u64, [u64, u64]),
            ("or_gl_mul", u64, [u64, u64]),
            ("or_gl_inv", u64, [u64]),
            ("or_ext2_mul", None, [_u64p, _u64p, _u64p]),
            ("or_ext2_inv", None, [_u64p, _u64p]),
            ("or_poseidon2_permute", None, [_u64p]),
            ("or_poseidon2_compress", None, [_u64p, _u64p, _u64p]),
            ("or_transcript_size", sz, []),
            ("or_tr_new", None, [vp, _c.c_char_p, sz]),
            ("or_tr_append_u64", None, [vp, _c.c_char_p, sz, u64]),
            ("or_tr_append_scalar", None, [vp, _c.c_char_p, sz, u64]),
            ("or_tr_append_ext2", None, [vp, _c.c_char_p, sz, _u64p]),
            ("or_tr_challenge_scalar", u64, [vp, _c.c_char_p, sz]),
            ("or_tr_challenge_ext2", None, [vp, _c.c_char_p, sz, _u64p]),
            ("or_sumcheck_prove_ext2", i32, [vp, i32, i32, _u64p, _u64p, _u64p, _u64p, _u64p]),
            ("or_sumcheck_prove_ext2_polys", i32, [vp, i32, i32, _u64p, _u64p, _u64p, _u64p, _u64p]),
            ("or_sumcheck_prove_base", i32, [vp, i32, i32, _u64p, _u64p, _u64p, _u64p, _u64p]),
            ("or_sumcheck_verify_ext2", i32, [vp, i32, i32, _u64p, _u64p, _u64p]),
            ("or_eq_table_base", None, [_u64p, i32, _u64p]),
            ("or_eq_table_ext2", None, [_u64p, i32, _u64p]),
            ("or_ml_eval_ext2", None, [_u64p, i32, _u64p, _u64p]),
            ("or_basefold_table_entries", sz, [i32, i32, i32]),
            ("or_basefold_table_generate", None, [i32, i32, i32, u64, _u64p, _u64p]),
            ("or_bhc_interpolate", None, [_u64p, i32, _u64p, _u64p]),
            ("or_basefold_encode", None, [_u64p, i32, i32, _u64p]),
            ("or_merkle_tree_gl", None, [_u64p, sz, _u64p]),
            ("or_merkle_tree_ext2", None, [_u64p, sz, _u64p]),
            ("or_basefold_commit", None, [_u64p, i32, i32, _u64p, _u64p, _u64p, _u64p]),
            ("or_basefold_proof_len", sz, [i32, i32, i32]),
            ("or_basefold_open_ext2", i32, [_u64p, _u64p, _u64p, _u64p, i32, i32, _u64p, _u64p, _u64p,
                                            vp, i32, _u64p]),
            ("or_basefold_verify_ext2", i32, [_u64p, i32, i32, _u64p, _u64p, i32, _u64p, _u64p, vp]),
            ("or_basefold_batch_proof_len", sz, [i32, i32, i32, i32]),
            ("or_basefold_batch_open_ext2", i32, [vp, vp, vp, _u64p, i32, i32, i32, _u64p, i32, _i32p, _i32p, _u64p,
                                                  i32, _u64p, _u64p, vp, i32, _u64p]),
            ("or_basefold_batch_verify_ext2", i32, [_u64p, i32, i32, i32, _u64p, i32, _i32p, _i32p, _u64p, i32,
                                                    _u64p, i32, _u64p, _u64p, vp]),
            ("or_partial_eval_base", None, [i32, _u64p, i32, _u64p, i32, _u64p]),
            ("or_partial_eval_ext2", None, [i32, _u64p, i32, _u64p, i32, _u64p]),
            ("or_bit_permute", None, [_u64p, _u64p, _i32p, i32]),
            ("or_fused_permute_peval", None, [i32, _u64p, i32, i32, i32, _u64p, _u32p, _u32p, _u64p]),
            ("or_agl_add", u64, [u64, u64]),
            ("or_agl_sub", u64, [u64, u64]),
            ("or_agl_mul", u64, [u64, u64]),
            ("or_aext2_mul", None, [_u64p, _u64p, _u64p]),
            ("or_monolith_permute", None, [_u64p]),
            ("or_monolith_tree_gl", None, [_u64p, ctypes.c_size_t, _u64p]),
            ("or_monolith_tree_ext2", None, [_u64p, ctypes.c_size_t, _u64p]),
            ("or_chacha8_block", None, [_u32p, _c.c_uint32, _u32p, _u32p]),
            ("or_ajtai_ring_elem", None, [_u32p, _c.c_uint32, u64, _u64p]),
            ("or_ajtai_commit_wide", None, [_u32p, _u64p, u64, u64, i32, i32, _u64p]),
            ("or_ajtai_commit_u8_batch", None, [_u32p, _u8p, u64, i32, i32, i32, _u64p]),
        ]:
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _LIB = L
    return _LIB


def ref_lib():
    """The reference's own Ajtai CPU code (host build), or None when not built."""
    global _REF
    if _REF is None:
        path = os.path.join(_HERE, "_ref", "libajtai_ref.so")
        if not os.path.exists(path):
            return None
        R = ctypes.CDLL(path)
        R.ref_chacha8_block.argtypes = [_u32p, _c.c_uint32, _u32p, _u32p]
        R.ref_ring_elem.argtypes = [_u32p, _c.c_int, _c.c_uint64, _u64p]
        R.ref_commit_wide.argtypes = [_u32p, _u64p, _c.c_uint64, _c.c_uint64, _c.c_int, _c.c_int, _u64p]
        R.ref_commit_binary.argtypes = [_u32p, _u64p, _c.c_uint64, _u64p]
        _REF = R
    return _REF


def set_threads(k):
    """Host threads for the large loops of one proof (results do not depend on them)."""
    lib().or_set_threads(int(k))


def get_threads():
    return int(lib().or_get_threads())


def _a(x, dt=np.uint64):
    return np.ascontiguousarray(np.asarray(x, dtype=dt))


class Transcript:
    """zk-torch-3 Transcript (transcript.rs:174-350)."""

    def __init__(self, label=b""):
        self.buf = ctypes.create_string_buffer(lib().or_transcript_size())
        lib().or_tr_new(self.buf, label, len(label))

    @property
    def ptr(self):
        return ctypes.cast(self.buf, ctypes.c_void_p)

    def append_u64(self, label, v):
        lib().or_tr_append_u64(self.ptr, label, len(label), int(v))

    def append_scalar(self, label, v):
        lib().or_tr_append_scalar(self.ptr, label, len(label), int(v))

    def append_ext2(self, label, v):
        lib().or_tr_append_ext2(self.ptr, label, len(label), _a(v))

    def challenge_scalar(self, label):
        return int(lib().or_tr_challenge_scalar(self.ptr, label, len(label)))

    def challenge_ext2(self, label):
        out = np.zeros(2, np.uint64)
        lib().or_tr_challenge_ext2(self.ptr, label, len(label), out)
        return out

    def state_bytes(self):
        return bytes(self.buf.raw)


def aext2_mul(a, b):
    """almost-Goldilocks Ext2 product (X^2 = 3), pinned to the reference's golden vectors."""
    out = np.zeros(2, np.uint64)
    lib().or_aext2_mul(_a(a), _a(b), out)
    return out


def monolith_permute(state):
    s = _a(state).copy()
    lib().or_monolith_permute(s)
    return s


def monolith_tree_gl(cw):
    cw = _a(cw)
    leaves = cw.size // 2
    tree = np.zeros((2 * leaves - 1) * 4, np.uint64)
    lib().or_monolith_tree_gl(cw, leaves, tree)
    return tree


def monolith_tree_ext2(cw):
    cw = _a(cw).reshape(-1)
    leaves = cw.size // 4
    tree = np.zeros((2 * leaves - 1) * 4, np.uint64)
    lib().or_monolith_tree_ext2(cw, leaves, tree)
    return tree


def poseidon2_permute(state):
    s = _a(state).copy()
    lib().or_poseidon2_permute(s)
    return s


def sumcheck_prove_ext2(transcript, polys):
    polys = _a(polys)
    d, N = polys.shape
    n = N.bit_length() - 1
    msgs = np.zeros((n, d + 1, 2), np.uint64)
    ch = np.zeros((n, 2), np.uint64)
    finals = np.zeros((d, 2), np.uint64)
    fe = np.zeros(2, np.uint64)
    rc = lib().or_sumcheck_prove_ext2(transcript.ptr, n, d, polys.reshape(-1), msgs.reshape(-1),
                                      ch.reshape(-1), finals.reshape(-1), fe)
    assert rc == 0
    return {"round_messages": msgs, "challenges": ch, "final_evals": finals, "final_eval": fe}


def sumcheck_prove_ext2_polys(transcript, polys):
    """polys: [d][2^n][2] Ext2 values."""
    polys = _a(polys)
    d, N = polys.shape[0], polys.shape[1]
    n = N.bit_length() - 1
    msgs = np.zeros((n, d + 1, 2), np.uint64)
    ch = np.zeros((n, 2), np.uint64)
    finals = np.zeros((d, 2), np.uint64)
    fe = np.zeros(2, np.uint64)
    rc = lib().or_sumcheck_prove_ext2_polys(transcript.ptr, n, d, polys.reshape(-1), msgs.reshape(-1),
                                            ch.reshape(-1), finals.reshape(-1), fe)
    assert rc == 0
    return {"round_messages": msgs, "challenges": ch, "final_evals": finals, "final_eval": fe}


def sumcheck_prove_base(transcript, polys):
    polys = _a(polys)
    d, N = polys.shape
    n = N.bit_length() - 1
    msgs = np.zeros((n, d + 1), np.uint64)
    ch = np.zeros(n, np.uint64)
    finals = np.zeros(d, np.uint64)
    fe = np.zeros(1, np.uint64)
    rc = lib().or_sumcheck_prove_base(transcript.ptr, n, d, polys.reshape(-1), msgs.reshape(-1), ch,
                                      finals, fe)
    assert rc == 0
    return {"round_messages": msgs, "challenges": ch, "final_evals": finals, "final_eval": fe}


def sumcheck_verify_ext2(transcript, n, d, claimed, msgs, final_eval):
    return bool(lib().or_sumcheck_verify_ext2(transcript.ptr, n, d, _a(claimed), _a(msgs).reshape(-1),
                                              _a(final_eval)))


def eq_table_ext2(point):
    point = _a(point).reshape(-1, 2)
    n = point.shape[0]
    out = np.zeros((1 << n, 2), np.uint64)
    lib().or_eq_table_ext2(point.reshape(-1), n, out.reshape(-1))
    return out


def ml_eval_ext2(evals, point):
    evals = _a(evals)
    n = evals.size.bit_length() - 1
    out = np.zeros(2, np.uint64)
    lib().or_ml_eval_ext2(evals, n, _a(point).reshape(-1), out)
    return out


def basefold_table(num_vars, log_rate, num_rounds, seed):
    tot = lib().or_basefold_table_entries(num_vars, log_rate, num_rounds)
    ent = np.zeros((tot, 2), np.uint64)
    off = np.zeros(num_rounds, np.uint64)
    lib().or_basefold_table_generate(num_vars, log_rate, num_rounds, seed, ent.reshape(-1), off)
    return ent, off


def bhc_interpolate(evals):
    evals = _a(evals)
    n = evals.size.bit_length() - 1
    co = np.zeros_like(evals)
    bh = np.zeros_like(evals)
    lib().or_bhc_interpolate(evals, n, co, bh)
    return co, bh


def basefold_encode(coeffs, log_rate):
    coeffs = _a(coeffs)
    n = coeffs.size.bit_length() - 1
    cw = np.zeros(coeffs.size << log_rate, np.uint64)
    lib().or_basefold_encode(coeffs, n, log_rate, cw)
    return cw


def merkle_tree_gl(cw):
    cw = _a(cw)
    leaves = cw.size // 2
    tree = np.zeros((2 * leaves - 1) * 4, np.uint64)
    lib().or_merkle_tree_gl(cw, leaves, tree)
    return tree


def merkle_tree_ext2(cw):
    cw = _a(cw).reshape(-1)
    leaves = cw.size // 4
    tree = np.zeros((2 * leaves - 1) * 4, np.uint64)
    lib().or_merkle_tree_ext2(cw, leaves, tree)
    return tree


def basefold_commit(evals, log_rate):
    evals = _a(evals)
    n = evals.size.bit_length() - 1
    cw = np.zeros(evals.size << log_rate, np.uint64)
    bh = np.zeros_like(evals)
    tree = np.zeros((2 * (cw.size // 2) - 1) * 4, np.uint64)
    root = np.zeros(4, np.uint64)
    lib().or_basefold_commit(evals, n, log_rate, cw, bh, tree, root)
    return {"root": root, "codeword": cw, "bh_evals": bh, "tree": tree, "num_vars": n, "log_rate": log_rate}


def basefold_proof_len(n, log_rate, q):
    return lib().or_basefold_proof_len(n, log_rate, q)


def basefold_open_ext2(comm, point, table, transcript, num_queries):
    n, lr = comm["num_vars"], comm["log_rate"]
    ent, off = table
    proof = np.zeros(basefold_proof_len(n, lr, num_queries), np.uint64)
    rc = lib().or_basefold_open_ext2(comm["codeword"], comm["bh_evals"], comm["tree"], comm["root"], n, lr,
                                     _a(point).reshape(-1), ent.reshape(-1), off, transcript.ptr,
                                     num_queries, proof)
    assert rc == 0
    return proof


def basefold_verify_ext2(root, n, log_rate, point, proof, num_queries, table, transcript):
    ent, off = table
    return bool(lib().or_basefold_verify_ext2(_a(root), n, log_rate, _a(point).reshape(-1), _a(proof),
                                              num_queries, ent.reshape(-1), off, transcript.ptr))


def basefold_batch_proof_len(n, log_rate, q, num_evals):
    return lib().or_basefold_batch_proof_len(n, log_rate, q, num_evals)


def _evals_arrays(evals):
    poly = _a([e[0] for e in evals], np.int32)
    point = _a([e[1] for e in evals], np.int32)
    vals = _a([np.asarray(e[2], np.uint64) for e in evals]).reshape(-1)
    return poly, point, vals


def basefold_batch_open_ext2(comms, points, evals, table, transcript, num_queries):
    """batch_open_ext2: comms are basefold_commit dicts, points a list of n-long Ext2 arrays,
    evals a list of (poly, point, value) with value an Ext2 pair."""
    n, lr = comms[0]["num_vars"], comms[0]["log_rate"]
    ent, off = table
    keep = [(_a(c["codeword"]), _a(c["bh_evals"]), _a(c["tree"])) for c in comms]
    ptrs = [(_c.c_void_p * len(comms))(*[k[j].ctypes.data for k in keep]) for j in range(3)]
    roots = _a([c["root"] for c in comms]).reshape(-1)
    pts = _a(points).reshape(-1)
    poly, point, vals = _evals_arrays(evals)
    proof = np.zeros(basefold_batch_proof_len(n, lr, num_queries, len(evals)), np.uint64)
    rc = lib().or_basefold_batch_open_ext2(_c.cast(ptrs[0], _c.c_void_p), _c.cast(ptrs[1], _c.c_void_p),
                                           _c.cast(ptrs[2], _c.c_void_p), roots, len(comms), n, lr, pts, len(points),
                                           poly, point, vals, len(evals), ent.reshape(-1), off, transcript.ptr,
                                           num_queries, proof)
    assert rc == 0
    return proof


def basefold_batch_verify_ext2(roots, n, log_rate, points, evals, proof, num_queries, table, transcript):
    ent, off = table
    poly, point, vals = _evals_arrays(evals)
    roots = _a(roots).reshape(-1)
    return bool(lib().or_basefold_batch_verify_ext2(roots, roots.size // 4, n, log_rate, _a(points).reshape(-1),
                                                    len(points), poly, point, vals, len(evals), _a(proof),
                                                    num_queries, ent.reshape(-1), off, transcript.ptr))


_FIELD = {"gl": 0, "agl": 1}


def partial_eval_base(evals, r, field="gl"):
    evals = _a(evals)
    log_n = evals.size.bit_length() - 1
    r = _a(r).reshape(-1)
    out = np.zeros(1 << (log_n - r.size), np.uint64)
    lib().or_partial_eval_base(_FIELD[field], evals, log_n, r if r.size else np.zeros(1, np.uint64), r.size, out)
    return out


def partial_eval_ext2(evals, r, field="gl"):
    evals = _a(evals)
    log_n = evals.size.bit_length() - 1
    r = _a(r).reshape(-1, 2)
    out = np.zeros((1 << (log_n - r.shape[0]), 2), np.uint64)
    lib().or_partial_eval_ext2(_FIELD[field], evals, log_n, r.reshape(-1), r.shape[0], out.reshape(-1))
    return out


def bit_permute(x, inv):
    x = _a(x)
    out = np.zeros_like(x)
    lib().or_bit_permute(x, out, _a(inv, np.int32), len(inv))
    return out


def fused_permute_peval(evals, n, m, half, eq, lo, hi, field="gl"):
    out = np.zeros((1 << (n - m), 2), np.uint64)
    lib().or_fused_permute_peval(_FIELD[field], _a(evals), n, m, half, _a(eq).reshape(-1), _a(lo, np.uint32),
                                 _a(hi, np.uint32), out.reshape(-1))
    return out


# ---- Ajtai fold-tree operations (cuda_almost_goldilocks/ajtai.cuh:700-1260), numpy restatement ----
def negacyclic_matrix(r):
    """T with (r . z)[k] = sum_l z[l] T[l, k]: T[l, k] = r[(k - l) mod 64], negated when l > k."""
    r = np.asarray(r, np.int64)
    l = np.arange(64)[:, None]
    k = np.arange(64)[None, :]
    idx = (k - l) % 64
    return np.where(l > k, -r[idx], r[idx])


def bits64(words):
    """[N] u64 -> [N, 64] int64 bits (bit l of word j at [j, l])."""
    w = np.asarray(words, np.uint64).reshape(-1)
    return ((w[:, None] >> np.arange(64, dtype=np.uint64)[None, :]) & np.uint64(1)).astype(np.int64)


def ajtai_multifold_mixed(zb, pos, neg, r_all):
    """multifold_mixed_witness_kernel (ajtai.cuh:1040-1122): zb [nb][N], pos/neg [nt][N] u64 masks,
    r_all [(nb + nt)][64] int8 -> [N][64] int16 (the i32 sum cast to i16)."""
    zb = np.asarray(zb, np.uint64).reshape(-1, np.asarray(zb).shape[-1]) if len(zb) else np.zeros((0, 0), np.uint64)
    r_all = np.asarray(r_all, np.int64).reshape(-1, 64)
    n = zb.shape[1] if zb.size else np.asarray(pos).shape[-1]
    acc = np.zeros((n, 64), np.int64)
    nb = zb.shape[0] if zb.size else 0
    for i in range(nb):
        acc += bits64(zb[i]) @ negacyclic_matrix(r_all[i])
    for t in range(len(pos)):
        acc += (bits64(pos[t]) - bits64(neg[t])) @ negacyclic_matrix(r_all[nb + t])
    return acc.astype(np.int16)


def ajtai_fold_witness(z1, z2, r):
    """fold_witness_kernel (ajtai.cuh:715-760): z1 + r . z2 in F_q, canonical [N][64]."""
    acc = bits64(z1) + bits64(z2) @ negacyclic_matrix(r)
    neg = acc < 0
    out = acc.astype(np.uint64)
    out[neg] = np.uint64(Q_AGL) - (-acc[neg]).astype(np.uint64)
    return out


def ajtai_split_witness(z):
    """split_witness_kernel (ajtai.cuh:1185-1243): [N][64] i16 -> pos, neg [13][N] u64."""
    z = np.asarray(z, np.int64).reshape(-1, 64)
    a = np.abs(z)
    pos = np.zeros((13, z.shape[0]), np.uint64)
    neg = np.zeros((13, z.shape[0]), np.uint64)
    w = (np.uint64(1) << np.arange(64, dtype=np.uint64))[None, :]
    for i in range(13):
        b = ((a >> i) & 1).astype(bool)
        pos[i] = np.bitwise_or.reduce(np.where(b & (z > 0), w, np.uint64(0)), axis=1)
        neg[i] = np.bitwise_or.reduce(np.where(b & (z < 0), w, np.uint64(0)), axis=1)
    return pos, neg


def ajtai_fold_commitments(c_first, c_all, r_all):
    """fold_commitment_kernel / multifold_commitment_kernel (ajtai.cuh:784-830, :1123-1147):
    c_first (or zero) + sum_i r_i . c_i over [KAPPA][64] rows of F_q, canonical."""
    c_all = [np.asarray(c, np.uint64).reshape(-1, 64) for c in c_all]
    out = np.zeros_like(c_all[0], dtype=object) if c_first is None else np.asarray(c_first, np.uint64).reshape(-1, 64).astype(object)
    for c, r in zip(c_all, np.asarray(r_all, np.int64).reshape(-1, 64)):
        T = negacyclic_matrix(r).astype(object)
        out = out + c.astype(object) @ T
    return (out % Q_AGL).astype(np.uint64)


def ajtai_ring_elem(key, row, j):
    out = np.zeros(64, np.uint64)
    lib().or_ajtai_ring_elem(_a(key, np.uint32), row, j, out)
    return out


def ajtai_commit_wide(key, z, col_offset=0, row_lo=0, nrows=42):
    z = _a(z).reshape(-1)
    N = z.size // 64
    out = np.zeros((nrows, 64), np.uint64)
    lib().or_ajtai_commit_wide(_a(key, np.uint32), z, N, col_offset, row_lo, nrows, out.reshape(-1))
    return out


def ajtai_commit_u8_batch(key, z8, row_lo=0, nrows=16):
    z8 = _a(z8, np.uint8)
    B = z8.shape[0]
    N = z8.shape[1] // 64
    out = np.zeros((B, nrows, 64), np.uint64)
    lib().or_ajtai_commit_u8_batch(_a(key, np.uint32), z8.reshape(-1), N, B, row_lo, nrows, out.reshape(-1))
    return out


# ---- The reference's own Basefold kernels run on the host (oracle/_ref/libbasefold_ref.so) ----
_REF_BF = None
_OBS = ctypes.CFUNCTYPE(None, ctypes.c_void_p, ctypes.POINTER(ctypes.c_uint64))
_SAMP = ctypes.CFUNCTYPE(ctypes.c_uint64, ctypes.c_void_p)


class _RefTranscript(ctypes.Structure):
    _fields_ = [("ctx", ctypes.c_void_p), ("observe_ext2", _OBS), ("observe_hash", _OBS), ("sample", _SAMP),
                ("sample_ext2", _OBS)]


def ref_basefold_lib():
    """The reference's Basefold/Merkle kernels built for the host, or None where the reference
    checkout was not available to build them."""
    global _REF_BF
    if _REF_BF is None:
        path = os.path.join(_HERE, "_ref", "libbasefold_ref.so")
        if not os.path.exists(path):
            return None
        R = ctypes.CDLL(path)
        R.ref_bf_init()
        R.ref_basefold_commit.argtypes = [_u64p, _c.c_int, _c.c_int, _u64p, _u64p, _u64p, _u64p]
        R.ref_merkle_tree_ext2.argtypes = [_u64p, _u64p, _c.c_int]
        R.ref_basefold_open_ext2.argtypes = [_u64p, _u64p, _u64p, _u64p, _c.c_int, _c.c_int, _u64p, _u64p, _u64p,
                                             ctypes.POINTER(_RefTranscript), _c.c_int, _u64p]
        _REF_BF = R
    return _REF_BF


def ref_basefold_commit(evals, log_rate):
    """BasefoldCommitment::commit_device made by the reference's kernels (canonical outputs)."""
    R = ref_basefold_lib()
    evals = _a(evals)
    n = evals.size.bit_length() - 1
    L = 1 << (n + log_rate)
    cw, bh = np.zeros(L, np.uint64), np.zeros(1 << n, np.uint64)
    tree, root = np.zeros((L - 1) * 4, np.uint64), np.zeros(4, np.uint64)
    R.ref_basefold_commit(evals, n, log_rate, cw, bh, tree, root)
    p = np.uint64(P)
    return {"root": root % p, "codeword": cw % p, "bh_evals": bh % p, "tree": tree % p, "num_vars": n,
            "log_rate": log_rate}


def ref_basefold_open_ext2(comm, point, table, transcript, num_queries):
    """open_ext2 (goldilocks-cuda-rs/src/basefold.rs:578-870) over the reference's kernels, the
    Fiat-Shamir steps on `transcript` (a Transcript of this package, the BasefoldTranscript rules of
    zk-torch-3/src/transcript.rs:331-350).  Returns the proof in the flat layout, canonical."""
    R = ref_basefold_lib()
    n, lr = comm["num_vars"], comm["log_rate"]
    ent, off = table
    t = transcript

    def observe_ext2(_, v):
        t.append_ext2(b"", np.array([v[0], v[1]], np.uint64))

    def observe_hash(_, h):
        for i in range(4):
            t.append_scalar(b"", h[i])

    def sample(_):
        return t.challenge_scalar(b"")

    def sample_ext2(_, out):
        c = t.challenge_ext2(b"")
        out[0], out[1] = int(c[0]), int(c[1])
    cbs = (_OBS(observe_ext2), _OBS(observe_hash), _SAMP(sample), _OBS(sample_ext2))
    rt = _RefTranscript(None, *cbs)
    proof = np.zeros(basefold_proof_len(n, lr, num_queries), np.uint64)
    rc = R.ref_basefold_open_ext2(_a(comm["codeword"]), _a(comm["bh_evals"]), _a(comm["tree"]), _a(comm["root"]), n,
                                  lr, _a(point).reshape(-1), _a(ent).reshape(-1), _a(off), ctypes.byref(rt),
                                  num_queries, proof)
    assert rc == 0
    return proof % np.uint64(P)


class _RefSumcheckTranscript(ctypes.Structure):
    _fields_ = [("ctx", ctypes.c_void_p), ("append_message", _OBS), ("challenge", _OBS)]


def ref_sumcheck_prove_ext2(transcript, polys):
    """GpuLinearSumcheckProver::new + prove (zk-torch-3/src/sumcheck/gpu_prover.rs:21-90) over the
    reference's sumcheck kernels (cuda/sumcheck_prover.cuh) run on the host; the transcript is a
    Transcript of this package.  Same result layout as sumcheck_prove_ext2."""
    R = ref_basefold_lib()
    R.ref_sumcheck_prove_ext2.argtypes = [_u64p, _c.c_int, _c.c_int, ctypes.POINTER(_RefSumcheckTranscript), _u64p,
                                          _u64p, _u64p, _u64p]
    polys = _a(polys)
    d, N = polys.shape
    n = N.bit_length() - 1
    t = transcript
    t.append_u64(b"num_var", n)
    t.append_u64(b"num_poly", d)

    def append_message(_, v):
        t.append_ext2(b"round_message", np.array([v[0], v[1]], np.uint64))

    def challenge(_, out):
        c = t.challenge_ext2(b"challenge")
        out[0], out[1] = int(c[0]), int(c[1])
    cbs = (_OBS(append_message), _OBS(challenge))
    rt = _RefSumcheckTranscript(None, *cbs)
    msgs = np.zeros((n, d + 1, 2), np.uint64)
    ch = np.zeros((n, 2), np.uint64)
    finals = np.zeros((d, 2), np.uint64)
    fe = np.zeros(2, np.uint64)
    rc = R.ref_sumcheck_prove_ext2(polys.reshape(-1), n, d, ctypes.byref(rt), msgs.reshape(-1), ch.reshape(-1),
                                   finals.reshape(-1), fe)
    assert rc == 0
    return {"round_messages": msgs, "challenges": ch, "final_evals": finals, "final_eval": fe}
