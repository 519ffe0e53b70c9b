"""Batched and served proving: every instance's proof equals its alone-run proof and the
oracle's composition (commit -> product sumcheck -> open of each polynomial at the
sumcheck point), whatever runs beside it."""
import numpy as np
import pytest

import oracle as O

pytestmark = pytest.mark.gpu
P = O.P
SEED = (0x1234567890ABCDEF % P, 0x0FEDCBA987654321 % P)
Q = 6
TABLE_NV = 12


@pytest.fixture(scope="module")
def tables(gpu_lib):
    from morpheus_gb300.basefold import BasefoldTable
    return BasefoldTable.generate(TABLE_NV, 1, TABLE_NV, 42), O.basefold_table(TABLE_NV, 1, TABLE_NV, 42)


def oracle_instance_proof(polys, index, q, table):
    """The instance protocol restated on the oracle (CPU)."""
    d, size = polys.shape
    n = size.bit_length() - 1
    comms = [O.basefold_commit(polys[j], 1) for j in range(d)]
    roots = np.stack([c["root"] for c in comms])
    t = O.Transcript(b"sumcheck")
    t.append_ext2(b"", np.array(SEED, np.uint64))
    t.append_u64(b"", index)
    for w in roots.reshape(-1):
        t.append_u64(b"", int(w))
    sc = O.sumcheck_prove_ext2(t, polys)
    opens = []
    for j in range(d):
        tj = O.Transcript(b"bf-open")
        tj.append_ext2(b"", np.array(SEED, np.uint64))
        tj.append_u64(b"", 8 * index + j)
        opens.append(O.basefold_open_ext2(comms[j], sc["challenges"], table, tj, q))
    return np.concatenate([roots.reshape(-1), sc["round_messages"].reshape(-1), sc["challenges"].reshape(-1),
                           sc["final_evals"].reshape(-1), sc["final_eval"].reshape(-1)] + opens)


def make(n, d, index, seed):
    from morpheus_gb300.batch import Instance
    rng = np.random.default_rng(seed)
    return Instance(rng.integers(0, P, size=(d, 1 << n), dtype=np.uint64), index, Q)


@pytest.mark.parametrize("n,d", [(2, 1), (3, 2), (6, 3), (9, 4), (12, 2)])
def test_instance_matches_oracle(tables, n, d):
    from morpheus_gb300 import batch
    gt, ot = tables
    inst = make(n, d, 7 + n, n * 10 + d)
    batch.prove_instance(gt, SEED, inst)
    want = oracle_instance_proof(inst.polys, inst.index, Q, ot)
    assert np.array_equal(inst.proof, want)
    # the open evaluations are the sumcheck's final evaluations, and the verifier accepts
    sp = inst.split()
    for j in range(d):
        assert np.array_equal(sp["opens"][j]["eval"], sp["final_evals"][j])
        tj = O.Transcript(b"bf-open")
        tj.append_ext2(b"", np.array(SEED, np.uint64))
        tj.append_u64(b"", 8 * inst.index + j)
        plen = O.basefold_proof_len(n, 1, Q)
        proof_j = inst.proof[-(d - j) * plen:][:plen]
        assert O.basefold_verify_ext2(sp["roots"][j], n, 1, sp["challenges"], proof_j, Q, ot, tj)


def test_batch_equals_alone_and_oracle(tables):
    from morpheus_gb300 import batch
    gt, ot = tables
    rng = np.random.default_rng(5)
    specs = [(int(rng.integers(2, TABLE_NV + 1)), int(rng.integers(1, 5))) for _ in range(24)]
    alone = [make(n, d, k, 100 + k) for k, (n, d) in enumerate(specs)]
    for inst in alone:
        batch.prove_instance(gt, SEED, inst)
    together = [make(n, d, k, 100 + k) for k, (n, d) in enumerate(specs)]
    batch.batch_prove(gt, SEED, together, workers=6)
    for a, b in zip(alone, together):
        assert np.array_equal(a.proof, b.proof)
    for inst in alone[:6]:
        assert np.array_equal(inst.proof, oracle_instance_proof(inst.polys, inst.index, Q, ot))


@pytest.mark.parametrize("budget", [1, 1 << 34])
def test_service_submit_wait(tables, budget):
    """A 1-byte budget admits one job at a time (each is larger than the budget); a large one
    runs them concurrently.  Results equal the alone runs either way."""
    from morpheus_gb300 import batch
    gt, _ = tables
    insts = [make(4 + k % 8, 1 + k % 4, 1000 + k, k) for k in range(12)]
    ref = []
    for inst in insts:
        r = make(inst.num_vars, inst.degree, inst.index, insts.index(inst))
        batch.prove_instance(gt, SEED, r)
        ref.append(r.proof.copy())
    with batch.ProverService(gt, SEED, Q, workers=4, hbm_budget=budget) as svc:
        tickets = [svc.submit(i) for i in insts]
        stats = []
        for t, want in zip(tickets, ref):
            inst, st = svc.wait(t)
            assert np.array_equal(inst.proof, want)
            assert st["latency_ms"] >= st["run_ms"] >= 0 and st["queued_ms"] >= 0
            stats.append(st)


def test_service_rejects_invalid(tables):
    from morpheus_gb300 import batch
    from morpheus_gb300 import _native as N
    gt, _ = tables
    with batch.ProverService(gt, SEED, Q, workers=2) as svc:
        bad = make(2, 1, 0, 0)
        bad.num_vars = 1  # n < 2 is not an instance
        with pytest.raises(N.NativeError, match="-2"):
            svc.submit(bad)
        with pytest.raises(N.NativeError):
            svc.wait(12345)  # unknown ticket


def test_mixed_workload_shapes(gpu_lib):
    from morpheus_gb300 import batch
    w = batch.mixed_workload(40, seed=3, min_vars=4, max_vars=9, num_queries=Q)
    assert {i.degree for i in w} <= {2, 3, 4}
    assert min(i.num_vars for i in w) >= 4 and max(i.num_vars for i in w) <= 9
    assert all(int(i.polys.max()) < P for i in w)


@pytest.mark.parametrize("coop,top", [(32768, 16), (0, 2), (1 << 40, 2048), (64, 256)])
def test_merkle_schedule_does_not_change_proofs(tables, coop, top):
    """The cooperative threshold and the single-CTA top size only change how the trees are
    scheduled (commit trees with replicated copies and every open round's tree)."""
    from morpheus_gb300 import batch
    gt, ot = tables
    inst = make(11, 2, 77, 4242)
    with batch.Schedule(coop, top):
        batch.prove_instance(gt, SEED, inst)
    assert np.array_equal(inst.proof, oracle_instance_proof(inst.polys, inst.index, Q, ot))


@pytest.mark.parametrize("budget,device", [(64 << 30, True), (1, False)])
def test_lockstep_engine_equals_alone(tables, budget, device):
    """The round-synchronous engine gives every instance its alone-run proof, in one wave or
    (1-byte budget) one instance per wave, from device or host inputs."""
    from morpheus_gb300 import batch
    gt, ot = tables
    rng = np.random.default_rng(21)
    specs = [(int(rng.integers(2, TABLE_NV + 1)), int(rng.integers(1, 5))) for _ in range(20)] + [(2, 1), (TABLE_NV, 4)]
    specs += [(3, 8), (6, 5)]  # the largest degrees of the sumcheck's lockstep kernels
    alone = [make(n, d, k, 300 + k) for k, (n, d) in enumerate(specs)]
    for inst in alone:
        batch.prove_instance(gt, SEED, inst)
    together = [make(n, d, k, 300 + k) for k, (n, d) in enumerate(specs)]
    if device:
        for inst in together:
            inst.to_device()
    batch.batch_prove(gt, SEED, together, workers=4, hbm_budget=budget, engine="lockstep")
    for a, b in zip(alone, together):
        assert np.array_equal(a.proof, b.proof)
    assert np.array_equal(alone[0].proof, oracle_instance_proof(alone[0].polys, alone[0].index, Q, ot))


@pytest.mark.parametrize("coop", [0, 1 << 40, 700])
def test_lockstep_layer_forms_do_not_change_proofs(tables, coop):
    """The lockstep committer's and open runner's Merkle layers give the same trees in each form:
    threshold 0 puts every layer in one permutation per thread (narrow CTAs for these small
    trees), 2^40 puts every layer in the 8-lane form, 700 mixes them within one proof."""
    from morpheus_gb300 import batch
    gt, _ = tables
    specs = [(TABLE_NV, 2), (12, 1), (9, 3), (5, 1), (TABLE_NV - 1, 1), (3, 2)]
    alone = [make(n, d, k, 500 + k) for k, (n, d) in enumerate(specs)]
    for inst in alone:
        batch.prove_instance(gt, SEED, inst)
    together = [make(n, d, k, 500 + k) for k, (n, d) in enumerate(specs)]
    batch.batch_prove(gt, SEED, together, workers=2, engine="lockstep", coop_threshold=coop)
    for a, b in zip(alone, together):
        assert np.array_equal(a.proof, b.proof)


@pytest.mark.parametrize("groups,parts", [(1, 1), (3, 2), (4, 3), (8, 8)])
def test_lockstep_schedule_does_not_change_proofs(tables, groups, parts):
    """Staggered groups and open parts (the lockstep autotuner's knobs) leave every proof its
    alone-run proof, including more groups or parts than there are instances or polynomials; the
    calling thread's schedule is restored afterwards."""
    import ctypes
    from morpheus_gb300 import batch, _native as N
    gt, _ = tables
    specs = [(TABLE_NV, 2), (10, 3), (7, 1), (4, 2), (TABLE_NV - 2, 1)]
    alone = [make(n, d, k, 700 + k) for k, (n, d) in enumerate(specs)]
    for inst in alone:
        batch.prove_instance(gt, SEED, inst)
    together = [make(n, d, k, 700 + k) for k, (n, d) in enumerate(specs)]
    batch.batch_prove(gt, SEED, together, workers=1, engine="lockstep", groups=groups, open_parts=parts)
    for a, b in zip(alone, together):
        assert np.array_equal(a.proof, b.proof)
    g, p = ctypes.c_int(), ctypes.c_int()
    N.lib().gb_get_lockstep_schedule(ctypes.byref(g), ctypes.byref(p))
    assert (g.value, p.value) == (2, 2)


def test_lockstep_schedule_rejects_out_of_range(gpu_lib):
    from morpheus_gb300 import _native as N
    L = N.lib()
    for g, p in [(0, 1), (1, 0), (9, 1), (1, 9)]:
        assert L.gb_set_lockstep_schedule(g, p) == -2
    assert L.gb_set_lockstep_schedule(2, 2) == 0
