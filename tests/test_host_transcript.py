"""The library's host transcript (branch-free Poseidon2 duplex) against the oracle's, on CPU.

Every challenge of the proof drivers comes from this transcript: a mixed sequence of labelled
appends and challenges, over random and edge-case field words, must leave both transcripts with
the same challenges and byte-identical states."""
import numpy as np
import pytest

P = 0xFFFFFFFF00000001
EDGE = [0, 1, P - 1, P, P + 1, 2**64 - 1, 2**32 - 1, 2**32, 2**63]


@pytest.fixture(scope="module")
def lib():
    from morpheus_gb300 import build as B
    B.build()
    from morpheus_gb300 import _native
    return _native.lib()


@pytest.mark.parametrize("seed", [1, 2, 3])
def test_transcript_matches_oracle(lib, seed):
    import oracle as O
    from morpheus_gb300.sumcheck import Transcript
    rng = np.random.default_rng(seed)
    labels = [b"", b"challenge", b"round_message", b"num_var", b"x"]
    t, o = Transcript(b"host-transcript"), O.Transcript(b"host-transcript")
    for step in range(400):
        word = lambda: int(EDGE[rng.integers(len(EDGE))]) if rng.random() < 0.3 else int(rng.integers(0, 2**64, dtype=np.uint64))
        label = labels[rng.integers(len(labels))]
        op = rng.integers(3)
        if op == 0:
            v = word()
            t.append_u64(label, v)
            o.append_u64(label, v)
        elif op == 1:
            v = [word() % P, word() % P]
            t.append_ext2(label, v)
            o.append_ext2(label, v)
        else:
            assert np.array_equal(t.challenge_ext2(label), o.challenge_ext2(label)), step
    assert t.state_bytes() == o.state_bytes()
