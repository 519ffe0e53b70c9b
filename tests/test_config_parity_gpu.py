"""Bit-exact parity at the configuration sizes, through the C ABI.

C1: the product sumcheck over 2 x 2^20 in both modes (Ext2 challenges, as GpuLinearSumcheckProver
and the verifier; base field, as LinearSumcheckProver), compared whole with the oracle on the same
inputs: every round message, challenge, final evaluation and the final product.

C2: Basefold commit + open_ext2 at 2^22 evaluations, rate 1/2, 34 queries, table (22, 1, 22, 42),
compared with the oracle's outputs recorded in tests/golden/config_goldens.json: root, codeword,
the whole tree, table entries and level offsets, and the entire proof.  The reference's own check
of the same kind is its GPU-against-CPU opening test (zk-torch-3/src/commit/cpu_basefold.rs:427-509).
"""
import hashlib
import json
import os

import numpy as np
import pytest

import oracle as O
import seeded_inputs as SI

pytestmark = pytest.mark.gpu
HERE = os.path.dirname(os.path.abspath(__file__))


def sha(a):
    return hashlib.sha256(np.ascontiguousarray(a, dtype="<u8").tobytes()).hexdigest()


@pytest.fixture(scope="module")
def goldens():
    with open(os.path.join(HERE, "golden", "config_goldens.json")) as f:
        return json.load(f)


@pytest.fixture(scope="module")
def c1():
    return SI.c1_polys()


def _check_sumcheck(pr, ref):
    assert np.array_equal(pr.round_messages, ref["round_messages"])
    assert np.array_equal(pr.challenges, ref["challenges"])
    assert np.array_equal(pr.final_evals, ref["final_evals"])
    assert np.array_equal(pr.final_eval.reshape(-1), np.asarray(ref["final_eval"]).reshape(-1))


@pytest.mark.parametrize("resident", [False, True])
def test_c1_sumcheck_ext2_2x2e20_bit_exact(gpu_lib, c1, resident):
    from morpheus_gb300 import sumcheck as S
    from morpheus_gb300.memory import DeviceBuffer
    n, d = SI.C1["num_vars"], SI.C1["degree"]
    ref = O.sumcheck_prove_ext2(O.Transcript(SI.C1["label"]), c1)
    t = S.Transcript(SI.C1["label"])
    if resident:
        buf = DeviceBuffer.from_numpy(c1.reshape(-1))
        pr = S.GpuLinearSumcheckProver(n, d, t).prove((buf, d), t)
        assert np.array_equal(buf.to_numpy(), c1.reshape(-1))  # inputs untouched
        buf.free()
    else:
        pr = S.GpuLinearSumcheckProver(n, d, t).prove(c1, t)
    _check_sumcheck(pr, ref)
    # the transcripts continue identically after the proof
    to = O.Transcript(SI.C1["label"])
    O.sumcheck_prove_ext2(to, c1)
    assert np.array_equal(t.challenge_ext2(b"after"), to.challenge_ext2(b"after"))


def test_c1_sumcheck_base_2x2e20_bit_exact(gpu_lib, c1):
    from morpheus_gb300 import sumcheck as S
    n, d = SI.C1["num_vars"], SI.C1["degree"]
    ref = O.sumcheck_prove_base(O.Transcript(SI.C1["label"]), c1)
    t = S.Transcript(SI.C1["label"])
    pr = S.LinearSumcheckProver(n, d, t).prove(c1, t)
    _check_sumcheck(pr, ref)


@pytest.mark.parametrize("key", ["c2", "c2_n16"])
def test_c2_basefold_commit_open_matches_oracle_fixture(gpu_lib, goldens, key):
    from morpheus_gb300 import sumcheck as S
    from morpheus_gb300.basefold import BasefoldCommitment, BasefoldTable
    g = goldens[key]
    n, lr, q = g["num_vars"], g["log_rate"], g["num_queries"]
    ev, pt = SI.c2_inputs(n)
    assert sha(ev) == g["evals_sha256"]
    table = BasefoldTable.generate(n, lr, n, g["table_seed"])
    assert sha(table.entries()) == g["table_entries_sha256"]
    assert [int(x) for x in table.level_offsets()] == g["table_level_offsets"]
    c = BasefoldCommitment.commit(ev, n, lr)
    assert [int(x) for x in c.root] == g["root"]
    tree = c.tree()
    top = len(g["tree_top_nodes"]) // 4
    assert [int(x) for x in tree.reshape(-1, 4)[-top:].reshape(-1)] == g["tree_top_nodes"]
    assert sha(tree) == g["tree_sha256"]
    assert sha(c.codeword()) == g["codeword_sha256"]
    proof = c.open_ext2(pt, table, S.Transcript(g["label"].encode()), q)
    assert proof.size == g["proof_len"]
    head = len(g["proof_head"])
    assert [int(x) for x in proof[:head]] == g["proof_head"]
    assert sha(proof) == g["proof_sha256"]
    # the same proof from evaluations already in device memory
    from morpheus_gb300.memory import DeviceBuffer
    d_ev = DeviceBuffer.from_numpy(ev)
    c2 = BasefoldCommitment.commit(d_ev, n, lr)
    assert [int(x) for x in c2.root] == g["root"]
    assert sha(c2.open_ext2(pt, table, S.Transcript(g["label"].encode()), q)) == g["proof_sha256"]
    d_ev.free()


def _ref_commit_cases():
    with open(os.path.join(HERE, "golden", "reference_basefold.json")) as f:
        return json.load(f)["basefold_commit_ref"]["cases"]


@pytest.mark.parametrize("case", _ref_commit_cases(), ids=lambda c: f"n{c['num_vars']}_lr{c['log_rate']}")
def test_commit_equals_reference_kernels(gpu_lib, case):
    """The commitment equals the one the reference's own Basefold and Merkle kernels made."""
    from morpheus_gb300.basefold import BasefoldCommitment
    n, lr = case["num_vars"], case["log_rate"]
    ev, _ = SI.c2_inputs(n)
    assert sha(ev) == case["evals_sha256"]
    c = BasefoldCommitment.commit(ev, n, lr)
    assert [int(x) for x in c.root] == case["root"]
    assert sha(c.codeword()) == case["codeword_sha256"]
    assert sha(c.tree()) == case["tree_sha256"]


def _ref_open_cases():
    with open(os.path.join(HERE, "golden", "reference_basefold.json")) as f:
        return json.load(f)["basefold_open_ref"]["cases"]


@pytest.mark.parametrize("case", _ref_open_cases(), ids=lambda c: c["name"])
def test_open_equals_reference_kernels(gpu_lib, case):
    """The whole proof equals the one open_ext2's sequence of the reference's own kernels made,
    including the exact inputs of the reference's GPU-against-CPU opening test
    (zk-torch-3/src/commit/cpu_basefold.rs:433-509: n = 6, table for 9 variables, rate 1/8)."""
    from morpheus_gb300 import sumcheck as S
    from morpheus_gb300.basefold import BasefoldCommitment, BasefoldTable
    n, lr, q = case["num_vars"], case["log_rate"], case["num_queries"]
    ev = np.array(case["evals"], np.uint64) if "evals" in case else SI.c2_inputs(n)[0]
    pt = np.array(case["point"], np.uint64).reshape(-1, 2)
    assert sha(ev) == case["evals_sha256"]
    c = BasefoldCommitment.commit(ev, n, lr)
    assert [int(x) for x in c.root] == case["root"]
    table = BasefoldTable.generate(case["table_vars"], lr, case["table_vars"], case["table_seed"])
    t = S.Transcript(case["label"].encode())
    if case["u64_after_label"] is not None:
        t.append_u64(b"", case["u64_after_label"])
    proof = c.open_ext2(pt, table, t, q)
    assert proof.size == case["proof_len"]
    assert [int(x) for x in proof[:len(case["proof_head"])]] == case["proof_head"]
    assert sha(proof) == case["proof_sha256"]


def _ref_sumcheck_cases():
    with open(os.path.join(HERE, "golden", "reference_basefold.json")) as f:
        return json.load(f)["sumcheck_ref"]["cases"]


@pytest.mark.parametrize("case", _ref_sumcheck_cases(), ids=lambda c: c["name"])
def test_sumcheck_equals_reference_kernels(gpu_lib, case):
    """Round messages, challenges and final evaluations equal those of the reference's own sumcheck
    kernels in GpuLinearSumcheckProver's sequence (c1 = the 2 x 2^20 configuration)."""
    from morpheus_gb300 import sumcheck as S
    d, n = case["degree"], case["num_vars"]
    polys = SI.field_elems(case["seed"], d << n).reshape(d, 1 << n)
    assert sha(polys) == case["polys_sha256"]
    t = S.Transcript(case["label"].encode())
    pr = S.GpuLinearSumcheckProver(n, d, t).prove(polys, t)
    assert [int(x) for x in pr.round_messages.reshape(-1)] == case["round_messages"]
    assert [int(x) for x in pr.challenges.reshape(-1)] == case["challenges"]
    assert [int(x) for x in pr.final_evals.reshape(-1)] == case["final_evals"]
    assert [int(x) for x in pr.final_eval.reshape(-1)] == case["final_eval"]
