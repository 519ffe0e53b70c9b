"""Batch opening (batch_open_ext2, goldilocks-cuda-rs/src/basefold.rs:1202-1532) on the GPU against
the oracle's restatement, on the reference's own test shapes (basefold.rs:3908-4170: num_vars 4,
log_rate 1, table seed 42, 4 queries; evaluations 1..16 and 100..115; points ((i+1) 111, (i+1) 222)
and ((i+1) 333, (i+1) 444)) and on larger random cases.  Every GPU proof is bit-identical to the
oracle's and the restated batch verifier (:1931-2220) accepts it."""
import numpy as np
import pytest

import oracle as O

P = O.P
pytestmark = pytest.mark.gpu


def ref_point(a, b, n):
    return np.array([[((i + 1) * a) % P, ((i + 1) * b) % P] for i in range(n)], np.uint64)


def run_case(evals_list, points, claims_of, n, lr, q, table_nv, label=b"bf-batch", seed_words=(5, 6)):
    """claims_of(evals_list, points) -> [(poly, point, value)]."""
    from morpheus_gb300.basefold import BasefoldCommitment, BasefoldTable, batch_open_ext2, split_batch_proof
    from morpheus_gb300.sumcheck import Transcript
    claims = claims_of(evals_list, points)
    table_h = O.basefold_table(table_nv, lr, table_nv, 42)
    ref_comms = [O.basefold_commit(ev, lr) for ev in evals_list]
    t = O.Transcript(label)
    t.append_ext2(b"", list(seed_words))
    ref = O.basefold_batch_open_ext2(ref_comms, points, claims, table_h, t, q)

    tab = BasefoldTable.generate(table_nv, lr, table_nv, 42)
    comms = [BasefoldCommitment.commit(ev, n, lr) for ev in evals_list]
    tg = Transcript(label)
    tg.append_ext2(b"", list(seed_words))
    proof = batch_open_ext2(comms, points, claims, tab, tg, q)
    assert np.array_equal(proof, ref)
    tv = O.Transcript(label)
    tv.append_ext2(b"", list(seed_words))
    roots = [c.root for c in comms]
    assert O.basefold_batch_verify_ext2(roots, n, lr, points, claims, proof, q, table_h, tv)
    assert np.array_equal(tg.challenge_ext2(b"x"), t.challenge_ext2(b"x"))
    return proof, split_batch_proof(proof, n, lr, q, len(claims)), claims, table_h, roots


def true_claims(pairs):
    def f(evals_list, points):
        return [(a, b, O.ml_eval_ext2(evals_list[a], points[b])) for a, b in pairs]
    return f


N4 = 4
EA = np.arange(1, 17, dtype=np.uint64)
EB = np.arange(100, 116, dtype=np.uint64)


def test_reference_single_poly(gpu_lib):
    run_case([EA], [ref_point(111, 222, N4)], true_claims([(0, 0)]), N4, 1, 4, N4)


def test_reference_two_polys_same_point(gpu_lib):
    run_case([EA, EB], [ref_point(111, 222, N4)], true_claims([(0, 0), (1, 0)]), N4, 1, 4, N4)


def test_reference_two_polys_different_points(gpu_lib):
    pts = [ref_point(111, 222, N4), ref_point(333, 444, N4)]
    proof, _, claims, table_h, roots = run_case([EA, EB], pts, true_claims([(0, 0), (1, 1)]), N4, 1, 4, N4)
    # the reference's tamper case (basefold.rs:4113-4170): a wrong claimed value is rejected
    bad = [(a, b, np.array([(int(v[0]) + 1) % P, int(v[1])], np.uint64)) if k == 0 else (a, b, v)
           for k, (a, b, v) in enumerate(claims)]
    tv = O.Transcript(b"bf-batch")
    tv.append_ext2(b"", [5, 6])
    assert not O.basefold_batch_verify_ext2(roots, N4, 1, pts, bad, proof, 4, table_h, tv)


@pytest.mark.parametrize("n,lr,q,npoly,pairs,table_nv", [
    (2, 1, 3, 1, [(0, 0)], 2),
    (5, 2, 6, 3, [(0, 0), (1, 1), (2, 0)], 6),                   # 3 claims: 2 weight bits, one unused weight
    (6, 1, 5, 2, [(0, 0), (1, 0), (1, 1), (0, 2), (1, 2)], 7),   # a polynomial at several points
    (9, 3, 10, 4, [(k, k % 2) for k in range(4)], 9),
    (12, 1, 34, 3, [(0, 0), (1, 1), (2, 1)], 12),
    (15, 1, 34, 2, [(0, 0), (1, 1)], 15),
])
def test_random_cases_match_oracle(gpu_lib, n, lr, q, npoly, pairs, table_nv):
    rng = np.random.default_rng(n * 100 + npoly)
    evals = [rng.integers(0, P, size=1 << n, dtype=np.uint64) for _ in range(npoly)]
    npts = max(b for _, b in pairs) + 1
    points = [rng.integers(0, P, size=(n, 2), dtype=np.uint64) for _ in range(npts)]
    _, sp, claims, _, _ = run_case(evals, points, true_claims(pairs), n, lr, q, table_nv)
    assert len(sp["combined_queries"]) == q and len(sp["individual_queries"][0]) == len(claims)


def test_invalid_arguments_rejected(gpu_lib):
    from morpheus_gb300 import _native as N
    from morpheus_gb300.basefold import BasefoldCommitment, BasefoldTable, batch_open_ext2
    from morpheus_gb300.sumcheck import Transcript
    tab = BasefoldTable.generate(5, 1, 5, 42)
    a = BasefoldCommitment.commit(np.arange(32, dtype=np.uint64), 5, 1)
    b = BasefoldCommitment.commit(np.arange(16, dtype=np.uint64), 4, 1)
    pt = [np.ones((5, 2), np.uint64)]
    v = np.zeros(2, np.uint64)
    for comms, claims in [([a], [(1, 0, v)]), ([a], [(0, 1, v)]), ([a, b], [(0, 0, v)]), ([a], [(-1, 0, v)])]:
        with pytest.raises(N.NativeError):
            batch_open_ext2(comms, pt, claims, tab, Transcript(b"x"), 2)
    small = BasefoldTable.generate(3, 1, 3, 42)  # does not cover num_vars 5
    with pytest.raises(N.NativeError):
        batch_open_ext2([a], pt, [(0, 0, v)], small, Transcript(b"x"), 2)
    assert N.lib().gb_basefold_batch_proof_len(5, 1, 2, 0) == 0
