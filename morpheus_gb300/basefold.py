"""Basefold commitment, mirroring goldilocks-cuda-rs/src/basefold.rs.

``BasefoldTable.generate`` / ``BasefoldCommitment.commit`` / ``open_ext2`` keep
the crate's names and argument meaning; the proof is returned in the flat
layout of gb_basefold_open_ext2 (include/goldilocks_cuda_wrapper.h), with
``split_proof`` giving the structured BasefoldProofExt2 view.
"""
import ctypes

import numpy as np

from . import _native as N
from .memory import DeviceBuffer


class BasefoldTable:
    """Folding table (BasefoldTable::generate + upload), device-resident."""

    def __init__(self, handle, num_vars, log_rate, num_rounds, seed):
        self.handle = handle
        self.num_vars, self.log_rate, self.num_rounds, self.seed = num_vars, log_rate, num_rounds, seed

    @classmethod
    def generate(cls, num_vars, log_rate, num_rounds, seed):
        h = ctypes.c_void_p()
        N.check(N.lib().gb_basefold_table_create(num_vars, log_rate, num_rounds, seed, ctypes.byref(h)),
                "gb_basefold_table_create")
        return cls(h, num_vars, log_rate, num_rounds, seed)

    def level_offsets(self):
        offs = np.zeros(self.num_rounds, np.uint64)
        ptr = ctypes.c_void_p()
        N.check(N.lib().gb_basefold_table_info(self.handle, ctypes.byref(ptr), offs.ctypes.data), "table_info")
        return offs

    def device_entries(self):
        ptr = ctypes.c_void_p()
        N.check(N.lib().gb_basefold_table_info(self.handle, ctypes.byref(ptr), None), "table_info")
        return ptr

    def device_level_ptr(self, level):
        return ctypes.c_void_p(self.device_entries().value + int(self.level_offsets()[level]) * 16)

    def entries(self):
        """Host copy of all (point, weight) entries, [total][2]."""
        sizes = [1 << (self.num_vars + self.log_rate - i - 1) for i in range(self.num_rounds)]
        total = sum(sizes)
        out = np.empty(total * 2, np.uint64)
        N.check(N.lib().cuda_memcpy_dtoh(out.ctypes.data, self.device_entries(), total * 16), "cuda_memcpy_dtoh")
        return out.reshape(total, 2)

    def __del__(self):
        try:
            if self.handle:
                N.lib().gb_basefold_table_destroy(self.handle)
                self.handle = None
        except Exception:
            pass


class BasefoldCommitment:
    """Device-resident commitment (codeword, Merkle tree, evaluations)."""

    def __init__(self, handle, num_vars, log_rate, root):
        self.handle = handle
        self.num_vars = num_vars
        self.log_rate = log_rate
        self.root = root

    @classmethod
    def commit(cls, evals, num_vars, log_rate):
        """evals: host array of 2^num_vars values, or a DeviceBuffer holding them."""
        h = ctypes.c_void_p()
        root = np.zeros(4, np.uint64)
        if isinstance(evals, DeviceBuffer):
            rc = N.lib().gb_basefold_commit(evals.ptr, None, num_vars, log_rate, ctypes.byref(h), root.ctypes.data)
        else:
            arr = np.ascontiguousarray(np.asarray(evals, dtype=np.uint64))
            assert arr.size == 1 << num_vars
            rc = N.lib().gb_basefold_commit(None, arr.ctypes.data, num_vars, log_rate, ctypes.byref(h),
                                            root.ctypes.data)
        N.check(rc, "gb_basefold_commit")
        return cls(h, num_vars, log_rate, root)

    commit_device = commit

    def _info(self):
        cw, tree, ev = ctypes.c_void_p(), ctypes.c_void_p(), ctypes.c_void_p()
        N.check(N.lib().gb_basefold_commitment_info(self.handle, ctypes.byref(cw), ctypes.byref(tree),
                                                    ctypes.byref(ev), None), "commitment_info")
        return cw, tree, ev

    def codeword(self):
        cw, _, _ = self._info()
        L = 1 << (self.num_vars + self.log_rate)
        out = np.empty(L, np.uint64)
        N.check(N.lib().cuda_memcpy_dtoh(out.ctypes.data, cw, L * 8), "cuda_memcpy_dtoh")
        return out

    def tree(self):
        _, tree, _ = self._info()
        leaves = (1 << (self.num_vars + self.log_rate)) // 2
        out = np.empty((2 * leaves - 1) * 4, np.uint64)
        N.check(N.lib().cuda_memcpy_dtoh(out.ctypes.data, tree, out.nbytes), "cuda_memcpy_dtoh")
        return out

    def open_ext2(self, point, table, transcript, num_queries):
        point = np.ascontiguousarray(np.asarray(point, dtype=np.uint64).reshape(-1))
        assert point.size == 2 * self.num_vars
        L = N.lib().gb_basefold_proof_len(self.num_vars, self.log_rate, num_queries)
        proof = np.zeros(L, np.uint64)
        rc = N.lib().gb_basefold_open_ext2(self.handle, table.handle, point.ctypes.data, ctypes.byref(transcript.state),
                                           num_queries, proof.ctypes.data)
        N.check(rc, "gb_basefold_open_ext2")
        return proof

    def __del__(self):
        try:
            if self.handle:
                N.lib().gb_basefold_commitment_destroy(self.handle)
                self.handle = None
        except Exception:
            pass


def split_proof(proof, n, lr, q):
    """Structured view of a flat proof (BasefoldProofExt2 field order)."""
    p = np.asarray(proof)
    o = 0
    eval_ = p[o:o + 2]
    o += 2
    oracles = p[o:o + n * 6].reshape(n, 3, 2)
    o += n * 6
    roots = p[o:o + (n - 1) * 4].reshape(n - 1, 4)
    o += (n - 1) * 4
    final = p[o:o + (2 << lr)].reshape(-1, 2)
    o += 2 << lr
    depths = [n + lr - 1 - r for r in range(n)]
    queries = []
    for _ in range(q):
        idx = int(p[o])
        o += 1
        vals = p[o:o + n * 4].reshape(n, 2, 2)
        o += n * 4
        paths = []
        for dpt in depths:
            paths.append(p[o:o + dpt * 4].reshape(dpt, 4))
            o += dpt * 4
        queries.append({"index": idx, "values": vals, "paths": paths})
    assert o == len(p)
    return {"eval": eval_, "oracles": oracles, "folded_roots": roots, "final_codeword": final, "queries": queries}


def batch_proof_len(num_vars, log_rate, num_queries, num_evals):
    return N.lib().gb_basefold_batch_proof_len(num_vars, log_rate, num_queries, num_evals)


def batch_open_ext2(comms, points, evals, table, transcript, num_queries):
    """batch_open_ext2 (goldilocks-cuda-rs/src/basefold.rs:1202-1532): open the commitments at Ext2
    points.  evals: (poly, point, value) triples, value an Ext2 pair; returns the flat proof
    (gb_basefold_batch_open_ext2 layout, see split_batch_proof)."""
    n, lr = comms[0].num_vars, comms[0].log_rate
    pts = np.ascontiguousarray(np.asarray(points, dtype=np.uint64).reshape(-1))
    assert pts.size == 2 * n * len(points)
    handles = (ctypes.c_void_p * len(comms))(*[c.handle for c in comms])
    poly = np.ascontiguousarray([e[0] for e in evals], dtype=np.int32)
    point = np.ascontiguousarray([e[1] for e in evals], dtype=np.int32)
    vals = np.ascontiguousarray(np.asarray([np.asarray(e[2], np.uint64) for e in evals], np.uint64).reshape(-1))
    L = batch_proof_len(n, lr, num_queries, max(len(evals), 1))
    proof = np.zeros(max(L, 1), np.uint64)
    rc = N.lib().gb_basefold_batch_open_ext2(ctypes.cast(handles, ctypes.c_void_p), len(comms), pts.ctypes.data,
                                             len(points), poly.ctypes.data, point.ctypes.data, vals.ctypes.data,
                                             len(evals), table.handle, ctypes.byref(transcript.state), num_queries,
                                             proof.ctypes.data)
    N.check(rc, "gb_basefold_batch_open_ext2")
    return proof


def split_batch_proof(proof, n, lr, q, num_evals):
    """Structured view of a flat batch proof (BatchBasefoldProofExt2 field order)."""
    p = np.asarray(proof)
    o = 0

    def take(k):
        nonlocal o
        v = p[o:o + k]
        o += k
        return v
    out = {"outer_oracles": take(n * 6).reshape(n, 3, 2), "combined_root": take(4), "inner_eval": take(2),
           "inner_oracles": take(n * 6).reshape(n, 3, 2), "folded_roots": take((n - 1) * 4).reshape(n - 1, 4),
           "final_codeword": take(2 << lr).reshape(-1, 2)}
    depths = [n + lr - 1 - r for r in range(n)]
    cq = []
    for _ in range(q):
        idx = int(take(1)[0])
        vals = take(n * 4).reshape(n, 2, 2)
        cq.append({"index": idx, "values": vals, "paths": [take(d * 4).reshape(d, 4) for d in depths]})
    iq = [[{"values": take(2), "path": take((n + lr - 1) * 4).reshape(-1, 4)} for _ in range(num_evals)]
          for _ in range(q)]
    assert o == len(p)
    out["combined_queries"] = cq
    out["individual_queries"] = iq
    return out
