"""Product sumcheck prover, mirroring zk-torch-3's prover interface.

``GpuLinearSumcheckProver`` keeps the reference's construction and call order
(zk-torch-3/src/sumcheck/gpu_prover.rs:13-89): the constructor appends
``num_var`` / ``num_poly`` to the transcript and ``prove`` returns a
``SumcheckProof`` (zk-torch-3/src/sumcheck/mod.rs:16-23).  The rounds run in the
CUDA library (gb_sumcheck_prove_ext2); only the transcript is on the host.
``LinearSumcheckProver`` is the base-field variant (linear_prover.rs:13-63).
"""
import ctypes
from dataclasses import dataclass

import numpy as np

from . import _native as N
from .memory import DeviceBuffer

P = 0xFFFFFFFF00000001


class Transcript:
    """zk-torch-3 Transcript (transcript.rs:174-350), state held in a gb_transcript."""

    def __init__(self, label=b""):
        self.state = N.GbTranscript()
        N.lib().gb_transcript_new(ctypes.byref(self.state), label)

    def append_u64(self, label, v):
        N.lib().gb_transcript_append_u64(ctypes.byref(self.state), label, int(v))

    def append_ext2(self, label, v):
        arr = (ctypes.c_uint64 * 2)(int(v[0]), int(v[1]))
        N.lib().gb_transcript_append_ext2(ctypes.byref(self.state), label, arr)

    def challenge_ext2(self, label):
        out = (ctypes.c_uint64 * 2)()
        N.lib().gb_transcript_challenge_ext2(ctypes.byref(self.state), label, out)
        return np.array([out[0], out[1]], np.uint64)

    def state_bytes(self):
        return bytes(self.state)


@dataclass
class SumcheckProof:
    final_eval: np.ndarray       # Ext2 [2] (or base [1])
    round_messages: np.ndarray   # [n][d+1][2] (or [n][d+1])
    challenges: np.ndarray
    final_evals: np.ndarray


def _prove(fn, transcript, polys, ext):
    if isinstance(polys, DeviceBuffer):
        raise TypeError("pass (DeviceBuffer, num_polys) as a tuple")
    if isinstance(polys, tuple):
        dbuf, d = polys
        n = (dbuf.len // d).bit_length() - 1
        dptr, hptr, keep = dbuf.ptr, None, None
    else:
        arr = np.ascontiguousarray(np.asarray(polys, dtype=np.uint64))
        d, size = arr.shape
        n = size.bit_length() - 1
        if size != 1 << n:
            raise ValueError("polynomial size must be a power of two")
        dptr, hptr, keep = None, ctypes.c_void_p(arr.ctypes.data), arr
    w = 2 if ext else 1
    msgs = np.zeros((n, d + 1, w) if ext else (n, d + 1), np.uint64)
    ch = np.zeros((n, w) if ext else (n,), np.uint64)
    finals = np.zeros((d, w) if ext else (d,), np.uint64)
    fe = np.zeros(w, np.uint64)
    rc = fn(ctypes.byref(transcript.state), n, d, dptr, hptr, msgs.ctypes.data, ch.ctypes.data, finals.ctypes.data,
            fe.ctypes.data)
    del keep
    N.check(rc, fn.__name__)
    return SumcheckProof(final_eval=fe, round_messages=msgs, challenges=ch, final_evals=finals)


class GpuLinearSumcheckProver:
    """Ext2-challenge product sumcheck (GpuLinearSumcheckProver::new / prove)."""

    def __init__(self, num_var, num_polys, transcript):
        self.num_var = num_var
        self.num_poly = num_polys
        self.challenges = None
        self.final_evals_ = None

    def prove(self, instances, transcript):
        """instances: [d][2^n] base-field values (numpy) or (DeviceBuffer, d)."""
        proof = _prove(N.lib().gb_sumcheck_prove_ext2, transcript, instances, True)
        self.challenges = proof.challenges
        self.final_evals_ = proof.final_evals
        return proof

    def final_eval(self, poly_idx):
        return self.final_evals_[poly_idx]


class LinearSumcheckProver:
    """Base-field product sumcheck (LinearSumcheckProver::new / prove)."""

    def __init__(self, num_var, num_polys, transcript):
        self.num_var = num_var
        self.num_poly = num_polys

    def prove(self, instances, transcript):
        return _prove(N.lib().gb_sumcheck_prove_base, transcript, instances, False)
