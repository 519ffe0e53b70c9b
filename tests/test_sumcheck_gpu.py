"""Product sumcheck on the GPU against the CPU oracle (bit-exact after canonicalisation)."""
import ctypes

import numpy as np
import pytest

import oracle as O

P = O.P
pytestmark = pytest.mark.gpu


def rand_polys(d, n, seed):
    return np.random.default_rng(seed).integers(0, P, size=(d, 1 << n), dtype=np.uint64)


@pytest.mark.parametrize("n,d", [(0, 2), (1, 1), (1, 2), (2, 2), (3, 3), (5, 2), (9, 4), (12, 2), (10, 8), (11, 5)])
def test_prove_ext2_matches_oracle(gpu_lib, n, d):
    from morpheus_gb300 import sumcheck as S
    polys = rand_polys(d, n, 1000 + 17 * n + d)
    ref = O.sumcheck_prove_ext2(O.Transcript(b"bench"), polys)
    t = S.Transcript(b"bench")
    pr = S.GpuLinearSumcheckProver(n, d, t).prove(polys, t)
    assert np.array_equal(pr.round_messages, ref["round_messages"])
    assert np.array_equal(pr.challenges, ref["challenges"])
    assert np.array_equal(pr.final_evals, ref["final_evals"])
    assert np.array_equal(pr.final_eval, ref["final_eval"])
    if n > 0:
        claim = int(ref["round_messages"][0, 0, 0]) + int(ref["round_messages"][0, 1, 0])
        assert O.sumcheck_verify_ext2(O.Transcript(b"bench"), n, d, [claim % P, 0], pr.round_messages, pr.final_eval)


@pytest.mark.parametrize("n,d", [(1, 2), (4, 3), (13, 2), (8, 6)])
def test_prove_base_matches_oracle(gpu_lib, n, d):
    from morpheus_gb300 import sumcheck as S
    polys = rand_polys(d, n, 77 + n + d)
    ref = O.sumcheck_prove_base(O.Transcript(b"test"), polys)
    t = S.Transcript(b"test")
    pr = S.LinearSumcheckProver(n, d, t).prove(polys, t)
    assert np.array_equal(pr.round_messages, ref["round_messages"])
    assert np.array_equal(pr.challenges, ref["challenges"])
    assert np.array_equal(pr.final_eval, ref["final_eval"])


def test_h70_hand_case(gpu_lib, golden):
    from morpheus_gb300 import sumcheck as S
    g = golden["sumcheck_h70"]
    polys = np.array([g["p1"], g["p2"]], np.uint64)
    t = S.Transcript(g["labels"]["ext2"].encode())
    pr = S.GpuLinearSumcheckProver(2, 2, t).prove(polys, t)
    assert (int(pr.round_messages[0, 0, 0]) + int(pr.round_messages[0, 1, 0])) % P == g["sum"]


def test_device_resident_input_and_transcript_state(gpu_lib):
    from morpheus_gb300 import sumcheck as S
    from morpheus_gb300.memory import DeviceBuffer
    polys = rand_polys(2, 14, 5)
    buf = DeviceBuffer.from_numpy(polys.reshape(-1))
    t1 = S.Transcript(b"x")
    p1 = S.GpuLinearSumcheckProver(14, 2, t1).prove((buf, 2), t1)
    t2 = S.Transcript(b"x")
    p2 = S.GpuLinearSumcheckProver(14, 2, t2).prove(polys, t2)
    assert np.array_equal(p1.round_messages, p2.round_messages)
    assert t1.state_bytes() == t2.state_bytes()
    # inputs untouched
    assert np.array_equal(buf.to_numpy(), polys.reshape(-1))
    # the transcript continues exactly like the oracle's after the proof
    to = O.Transcript(b"x")
    O.sumcheck_prove_ext2(to, polys)
    assert np.array_equal(t1.challenge_ext2(b"after"), to.challenge_ext2(b"after"))


def test_full_size_properties(gpu_lib):
    """2^20 x 2 (the bench shape): the verifier accepts and s_0(0)+s_0(1) is the claimed sum."""
    from morpheus_gb300 import sumcheck as S
    n, d = 20, 2
    polys = rand_polys(d, n, 2024)
    t = S.Transcript(b"bench")
    pr = S.GpuLinearSumcheckProver(n, d, t).prove(polys, t)
    claim = int((polys[0].astype(object) * polys[1].astype(object)).sum() % P)
    m = pr.round_messages
    assert (int(m[0, 0, 0]) + int(m[0, 1, 0])) % P == claim
    assert O.sumcheck_verify_ext2(O.Transcript(b"bench"), n, d, [claim, 0], m, pr.final_eval)


@pytest.mark.parametrize("ext", [False, True])
@pytest.mark.parametrize("d", [1, 2, 3])
def test_reference_ffi_round_and_fold(gpu_lib, ext, d):
    """sumcheck_round_message[_ext2]_ffi / sumcheck_fold[_ext2]_ffi with the reference's layout."""
    from morpheus_gb300.memory import DeviceBuffer
    L = gpu_lib
    n = 9
    N = 1 << n
    w = 2 if ext else 1
    rng = np.random.default_rng(d * 3 + ext)
    vals = rng.integers(0, P, size=(d, N, w), dtype=np.uint64)
    buf = DeviceBuffer.from_numpy(vals.reshape(-1))
    half = N // 2
    blocks = min((half + 255) // 256, 256)
    part = DeviceBuffer(blocks * (d + 1) * w)
    fn = L.sumcheck_round_message_ext2_ffi if ext else L.sumcheck_round_message_ffi
    assert fn(buf.ptr, part.ptr, d, N, half, blocks) == 0
    parts = part.to_numpy().reshape(blocks, d + 1, w).astype(object).sum(axis=0) % P
    # expected message from the definition
    A = vals.astype(object)

    def emul(a, b):
        if not ext:
            return (a[0] * b[0]) % P,
        return ((a[0] * b[0] + 7 * a[1] * b[1]) % P, (a[0] * b[1] + a[1] * b[0]) % P)

    for c in range(d + 1):
        acc = [0] * w
        for y in range(half):
            prod = tuple([1] + [0] * (w - 1))
            for i in range(d):
                e, o = A[i, 2 * y], A[i, 2 * y + 1]
                v = tuple((e[k] + c * (o[k] - e[k])) % P for k in range(w))
                prod = emul(prod, v)
            acc = [(acc[k] + prod[k]) % P for k in range(w)]
        assert [int(x) for x in parts[c]] == acc
    out = DeviceBuffer(d * N * w)
    r = [int(x) for x in rng.integers(0, P, size=2, dtype=np.uint64)]
    if ext:
        assert L.sumcheck_fold_ext2_ffi(buf.ptr, out.ptr, r[0], r[1], d, N, half) == 0
    else:
        assert L.sumcheck_fold_ffi(buf.ptr, out.ptr, r[0], d, N, half) == 0
    got = out.to_numpy().reshape(d, N, w)[:, :half].astype(object) % P
    for i in range(d):
        for y in range(0, half, 37):
            e, o = A[i, 2 * y], A[i, 2 * y + 1]
            diff = tuple((o[k] - e[k]) % P for k in range(w))
            rr = tuple(r[:w])
            pr = emul(rr, diff)
            assert [int(x) for x in got[i, y]] == [(e[k] + pr[k]) % P for k in range(w)]
