"""Served matmul-layer jobs: the proof equals the oracle's composition of the protocol, and
each job's proof is the same alone and when it runs beside others in the prover service."""
import numpy as np
import pytest

import oracle as O

pytestmark = pytest.mark.gpu
P = O.P
SEED = (0x0123456789ABCDEF % P, 0x7777777777777777 % P)
AJ_KEY = np.array([11, 22, 33, 44, 55, 66, 77, 88], np.uint32)
Q = 5
TABLE_NV = 16


@pytest.fixture(scope="module")
def env(gpu_lib):
    from morpheus_gb300.ajtai import AjtaiKey
    from morpheus_gb300.basefold import BasefoldTable
    return (BasefoldTable.generate(TABLE_NV, 1, TABLE_NV, 42), AjtaiKey(AJ_KEY, 0, 16, 1024),
            O.basefold_table(TABLE_NV, 1, TABLE_NV, 42))


def embed(x):
    x = x.astype(np.int64)
    out = x.astype(np.uint64)
    neg = x < 0
    out[neg] = np.uint64(P) - (-x[neg]).astype(np.uint64)
    return out


def ext_dot(eq, mat, axis):
    """sum over `axis` of eq (Ext2, [len][2]) times the base matrix, mod p -> [other][2]"""
    m = mat.astype(object)
    e0, e1 = eq[:, 0].astype(object), eq[:, 1].astype(object)
    if axis == 0:
        c0 = (e0[:, None] * m).sum(axis=0) % P
        c1 = (e1[:, None] * m).sum(axis=0) % P
    else:
        c0 = (m * e0[None, :]).sum(axis=1) % P
        c1 = (m * e1[None, :]).sum(axis=1) % P
    return np.stack([c0.astype(np.uint64), c1.astype(np.uint64)], -1)


def oracle_matmul_proof(a8, b8, index, q, table):
    m, k = a8.shape
    n = b8.shape[1]
    lm, ln, lk = m.bit_length() - 1, n.bit_length() - 1, k.bit_length() - 1
    A, B = embed(a8), embed(b8)
    ca, cb = O.basefold_commit(A.reshape(-1), 1), O.basefold_commit(B.reshape(-1), 1)
    t = O.Transcript(b"matmul")
    t.append_ext2(b"", np.array(SEED, np.uint64))
    for v in (index, m, n, k):
        t.append_u64(b"", v)
    for w in np.concatenate([ca["root"], cb["root"]]):
        t.append_u64(b"", int(w))
    pt = np.array([t.challenge_ext2(b"") for _ in range(lm + ln)], np.uint64).reshape(-1, 2)
    r_i, r_j = pt[:lm], pt[lm:]
    a = ext_dot(O.eq_table_ext2(r_i), A, axis=0)
    b = ext_dot(O.eq_table_ext2(r_j), B, axis=1)
    sc = O.sumcheck_prove_ext2_polys(t, np.stack([a, b]))
    m0 = sc["round_messages"][0]
    claim = np.array([(int(m0[0, 0]) + int(m0[1, 0])) % P, (int(m0[0, 1]) + int(m0[1, 1])) % P], np.uint64)
    r_k = sc["challenges"]
    opens = []
    for which, (comm, point) in enumerate([(ca, np.concatenate([r_k, r_i])), (cb, np.concatenate([r_j, r_k]))]):
        to = O.Transcript(b"bf-open")
        to.append_ext2(b"", np.array(SEED, np.uint64))
        to.append_u64(b"", 8 * index + which)
        opens.append(O.basefold_open_ext2(comm, point, table, to, q))
    w = (a8.reshape(-1)[:1 << 16].astype(np.int16) + 128).astype(np.uint8)
    aj = O.ajtai_commit_u8_batch(AJ_KEY, w[None, :], row_lo=0, nrows=16)
    return np.concatenate([ca["root"], cb["root"], claim, sc["round_messages"].reshape(-1), r_k.reshape(-1),
                           sc["final_evals"].reshape(-1), sc["final_eval"].reshape(-1), opens[0], opens[1],
                           aj.reshape(-1)]), (A, B, r_i, r_j, r_k)


def make(m, n, k, index, seed):
    from morpheus_gb300.batch import MatmulJob
    rng = np.random.default_rng(seed)
    return MatmulJob(rng.integers(-128, 128, size=(m, k), dtype=np.int8),
                     rng.integers(-128, 128, size=(k, n), dtype=np.int8), index, Q)


@pytest.mark.parametrize("m,n,k", [(256, 4, 256), (128, 2, 512)])
def test_matmul_job_matches_oracle(env, m, n, k):
    from morpheus_gb300 import batch
    gt, key, ot = env
    job = make(m, n, k, 3 + m, m + n + k)
    batch.prove_matmul(gt, key, SEED, job)
    want, (A, B, r_i, r_j, r_k) = oracle_matmul_proof(job.a, job.b, job.index, Q, ot)
    assert np.array_equal(job.proof, want)
    sp = job.split()
    # the claim is C~(r_i, r_j) of the product matrix, and the openings' evaluations are the
    # sumcheck's final values
    C = (A.astype(object) @ B.astype(object)) % P
    eq_i, eq_j = O.eq_table_ext2(r_i), O.eq_table_ext2(r_j)
    row = ext_dot(eq_i, C, axis=0)                   # [n][2]: sum_i eq_i C[i][j]
    c0 = sum(int(row[j, 0]) * int(eq_j[j, 0]) + 7 * int(row[j, 1]) * int(eq_j[j, 1]) for j in range(n)) % P
    c1 = sum(int(row[j, 0]) * int(eq_j[j, 1]) + int(row[j, 1]) * int(eq_j[j, 0]) for j in range(n)) % P
    assert [int(x) for x in sp["claim"]] == [c0, c1]
    la = O.basefold_proof_len(m.bit_length() - 1 + k.bit_length() - 1, 1, Q)
    assert np.array_equal(sp["open_a"][:2], sp["final_evals"][0])
    assert np.array_equal(sp["open_b"][:2], sp["final_evals"][1])
    assert sp["open_a"].size == la


def test_served_mix_equals_alone(env):
    """Matmul jobs and sumcheck instances submitted together to a 4-worker service give the
    proofs each gives alone."""
    from morpheus_gb300 import batch
    gt, key, _ = env
    jobs = [make(256, 16, 256, 100 + i, i) for i in range(3)] + [make(512, 8, 128, 200 + i, 50 + i) for i in range(3)]
    alone = []
    for j in jobs:
        batch.prove_matmul(gt, key, SEED, j)
        alone.append(j.proof.copy())
        j.proof[:] = 0
    rng = np.random.default_rng(9)
    insts = [batch.Instance(rng.integers(0, P, size=(2, 1 << 10), dtype=np.uint64), 500 + i, Q) for i in range(4)]
    inst_alone = []
    for i in insts:
        batch.prove_instance(gt, SEED, i)
        inst_alone.append(i.proof.copy())
        i.proof[:] = 0
    with batch.ProverService(gt, SEED, Q, workers=4, hbm_budget=8 << 30) as svc:
        svc.set_ajtai_key(key)
        tickets = [svc.submit(x) for pair in zip(jobs, insts + [None] * 2) for x in pair if x is not None]
        lat = [svc.wait(t)[1]["latency_ms"] for t in tickets]
    assert all(x > 0 for x in lat)
    for j, want in zip(jobs, alone):
        assert np.array_equal(j.proof, want)
    for i, want in zip(insts, inst_alone):
        assert np.array_equal(i.proof, want)


def test_matmul_job_rejects_bad_shapes(env):
    from morpheus_gb300 import batch
    from morpheus_gb300 import _native as N
    gt, key, _ = env
    with pytest.raises(ValueError):
        make(256, 3, 256, 0, 0)  # n not a power of two
    job = make(64, 4, 64, 0, 0)  # m k = 2^12 < 2^16: no 2^16-entry witness
    with pytest.raises(N.NativeError, match="-2"):
        batch.prove_matmul(gt, key, SEED, job)


@pytest.mark.parametrize("budget", [1, 8 << 30])
def test_continuous_service_mix_equals_alone(env, budget):
    """The continuous service (prologues on the workers, every opening in the open engines) gives
    each matmul job and each instance the proof it gives alone; a 1-byte budget admits one job
    at a time, a large one lets their openings share the engines' steps."""
    from morpheus_gb300 import batch
    gt, key, _ = env
    jobs = [make(256, 16, 256, 300 + i, 70 + i) for i in range(2)] + [make(512, 8, 128, 400 + i, 80 + i)
                                                                      for i in range(2)]
    rng = np.random.default_rng(19)
    insts = [batch.Instance(rng.integers(0, P, size=(1 + i % 3, 1 << (4 + 3 * i)), dtype=np.uint64), 600 + i, Q)
             for i in range(4)]
    alone = []
    for x in jobs + insts:
        (batch.prove_matmul(gt, key, SEED, x) if isinstance(x, batch.MatmulJob) else batch.prove_instance(gt, SEED, x))
        alone.append(x.proof.copy())
        x.proof[:] = 0
    with batch.ProverService(gt, SEED, Q, workers=3, hbm_budget=budget, continuous=True) as svc:
        svc.set_ajtai_key(key)
        order = [x for pair in zip(jobs, insts) for x in pair]
        tickets = [svc.submit(x) for x in order]
        stats = [svc.wait(t)[1] for t in tickets]
        assert svc.running() == 0 and svc.openings_in_flight() == 0
    assert all(st["latency_ms"] >= st["run_ms"] > 0 for st in stats)
    for x in order:
        assert np.array_equal(x.proof, alone[(jobs + insts).index(x)])


@pytest.mark.parametrize("coop", [0, 1 << 40])
def test_continuous_service_layer_forms_do_not_change_proofs(env, coop):
    """The open engines take the creating thread's cooperative threshold for their Merkle
    layers: 0 puts every layer in one permutation per thread, 2^40 every layer in the 8-lane
    form; the proofs are the alone-run proofs either way."""
    from morpheus_gb300 import batch
    gt, key, _ = env
    rng = np.random.default_rng(31)
    insts = [batch.Instance(rng.integers(0, P, size=(1 + i % 2, 1 << n), dtype=np.uint64), 900 + i, Q)
             for i, n in enumerate((TABLE_NV, 11, 7, 3))]
    jobs = [make(256, 16, 256, 950, 97)]
    alone = []
    for x in jobs + insts:
        (batch.prove_matmul(gt, key, SEED, x) if isinstance(x, batch.MatmulJob) else batch.prove_instance(gt, SEED, x))
        alone.append(x.proof.copy())
        x.proof[:] = 0
    with batch.Schedule(coop, None):
        svc = batch.ProverService(gt, SEED, Q, workers=2, hbm_budget=8 << 30, continuous=True)
    with svc:
        svc.set_ajtai_key(key)
        for t in [svc.submit(x) for x in jobs + insts]:
            svc.wait(t)
    for x, a in zip(jobs + insts, alone):
        assert np.array_equal(x.proof, a)


def test_continuous_service_jobs_join_openings_in_flight(env):
    """Jobs submitted while another job's openings are in the engines join their steps, and every
    proof is still its alone-run proof."""
    import time
    from morpheus_gb300 import batch
    gt, key, _ = env
    first = make(256, 64, 256, 700, 90)
    late = [make(256, 8, 256, 701 + i, 91 + i) for i in range(3)]
    rng = np.random.default_rng(23)
    late_insts = [batch.Instance(rng.integers(0, P, size=(2, 1 << 12), dtype=np.uint64), 800 + i, Q) for i in range(2)]
    alone = []
    for x in [first] + late + late_insts:
        (batch.prove_matmul(gt, key, SEED, x) if isinstance(x, batch.MatmulJob) else batch.prove_instance(gt, SEED, x))
        alone.append(x.proof.copy())
        x.proof[:] = 0
    with batch.ProverService(gt, SEED, Q, workers=2, hbm_budget=8 << 30, continuous=True) as svc:
        svc.set_ajtai_key(key)
        t0 = svc.submit(first)
        deadline = time.time() + 30
        while svc.openings_in_flight() == 0 and svc.running() > 0 and time.time() < deadline:
            time.sleep(0.0005)
        tickets = [t0] + [svc.submit(x) for x in late + late_insts]
        for t in tickets:
            svc.wait(t)
    for x, want in zip([first] + late + late_insts, alone):
        assert np.array_equal(x.proof, want)


def test_continuous_service_spans_size_classes(env):
    """Instances whose openings fall in each of the engines' size classes (2^12, 2^19 and 2^22
    evaluations) run together in the continuous service with their alone-run proofs."""
    from morpheus_gb300 import batch
    from morpheus_gb300.basefold import BasefoldTable
    _, key, _ = env
    gt = BasefoldTable.generate(22, 1, 22, 42)
    rng = np.random.default_rng(29)
    insts = [batch.Instance(rng.integers(0, P, size=(1, 1 << n), dtype=np.uint64), 900 + n, Q) for n in (22, 12, 19)]
    alone = []
    for x in insts:
        batch.prove_instance(gt, SEED, x)
        alone.append(x.proof.copy())
        x.proof[:] = 0
    with batch.ProverService(gt, SEED, Q, workers=3, hbm_budget=16 << 30, continuous=True) as svc:
        for t in [svc.submit(x) for x in insts]:
            svc.wait(t)
    for x, want in zip(insts, alone):
        assert np.array_equal(x.proof, want)


def test_continuous_service_slots_bound_jobs_in_flight(env):
    """With one job slot the continuous service never has more than one job admitted at a time,
    whatever the budget, and the proofs are still the alone-run ones."""
    import threading
    from morpheus_gb300 import batch
    gt, _, _ = env
    rng = np.random.default_rng(37)
    insts = [batch.Instance(rng.integers(0, P, size=(2, 1 << 11), dtype=np.uint64), 1000 + i, Q) for i in range(6)]
    alone = []
    for x in insts:
        batch.prove_instance(gt, SEED, x)
        alone.append(x.proof.copy())
        x.proof[:] = 0
    seen, stop = [], threading.Event()
    with batch.ProverService(gt, SEED, Q, workers=3, hbm_budget=8 << 30, continuous=True, slots=1) as svc:
        def watch():
            while not stop.is_set():
                seen.append(svc.running())
        th = threading.Thread(target=watch)
        th.start()
        try:
            for t in [svc.submit(x) for x in insts]:
                svc.wait(t)
        finally:
            stop.set()
            th.join()
    assert max(seen) <= 1
    for x, want in zip(insts, alone):
        assert np.array_equal(x.proof, want)
