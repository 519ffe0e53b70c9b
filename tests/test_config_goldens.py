"""The configuration fixtures (tests/golden/config_goldens.json) on CPU: the seeded inputs hash
to the recorded digests on this machine, and the oracle reproduces the n = 16 fixture whole."""
import hashlib
import json
import os

import numpy as np
import pytest

import oracle as O
import seeded_inputs as SI

HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.fixture(scope="module")
def goldens():
    with open(os.path.join(HERE, "golden", "config_goldens.json")) as f:
        return json.load(f)


def sha(a):
    return hashlib.sha256(np.ascontiguousarray(a, dtype="<u8").tobytes()).hexdigest()


def test_splitmix64_known_answers():
    # splitmix64 from state 0: the published first outputs of the generator
    assert [int(x) for x in SI.splitmix64(0, 3)] == [0xE220A8397B1DCDAF, 0x6E789E6AA1B965F4, 0x06C45D188009454F]


@pytest.mark.parametrize("key", ["c2", "c2_n16"])
def test_seeded_inputs_match_fixture(goldens, key):
    g = goldens[key]
    ev, pt = SI.c2_inputs(g["num_vars"])
    assert sha(ev) == g["evals_sha256"]
    assert [int(x) for x in pt.reshape(-1)] == g["point"]


def test_oracle_reproduces_n16_fixture(goldens):
    g = goldens["c2_n16"]
    n, lr, q = g["num_vars"], g["log_rate"], g["num_queries"]
    ev, pt = SI.c2_inputs(n)
    ent, off = O.basefold_table(n, lr, n, g["table_seed"])
    assert sha(ent) == g["table_entries_sha256"] and [int(x) for x in off] == g["table_level_offsets"]
    c = O.basefold_commit(ev, lr)
    assert [int(x) for x in c["root"]] == g["root"]
    assert sha(c["codeword"]) == g["codeword_sha256"] and sha(c["tree"]) == g["tree_sha256"]
    proof = O.basefold_open_ext2(c, pt, (ent, off), O.Transcript(g["label"].encode()), q)
    assert proof.size == g["proof_len"] and sha(proof) == g["proof_sha256"]
    assert [int(x) for x in proof[:len(g["proof_head"])]] == g["proof_head"]
