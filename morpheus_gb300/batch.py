"""Batched and served proving of many independent instances (native prover service).

An instance is ``degree`` multilinear polynomials of 2^num_vars Goldilocks values, proven by
Basefold commits, the product sumcheck, and one open_ext2 per polynomial at the sumcheck
point, on per-instance transcripts (the layout is documented beside ``gb_instance`` in
include/goldilocks_cuda_wrapper.h).  ``prove_instance`` is the per-call path;
``batch_prove`` and ``ProverService`` run many instances concurrently on worker threads with
a stream each, admitted against an HBM budget.  The worker count is tuned by ``autotune``.
"""
import ctypes
import time

import numpy as np

from . import _native as N
from .basefold import split_proof

P = 0xFFFFFFFF00000001
LOG_RATE = 1


class GbInstance(ctypes.Structure):
    _fields_ = [("num_vars", ctypes.c_int), ("degree", ctypes.c_int), ("index", ctypes.c_uint64),
                ("h_polys", ctypes.c_void_p), ("d_polys", ctypes.c_void_p), ("h_proof", ctypes.c_void_p)]


class GbMatmulJob(ctypes.Structure):
    _fields_ = [("m", ctypes.c_int), ("n", ctypes.c_int), ("k", ctypes.c_int), ("index", ctypes.c_uint64),
                ("h_a", ctypes.c_void_p), ("h_b", ctypes.c_void_p), ("h_proof", ctypes.c_void_p)]


class GbJobStats(ctypes.Structure):
    _fields_ = [("queued_ms", ctypes.c_double), ("run_ms", ctypes.c_double), ("latency_ms", ctypes.c_double)]


def instance_proof_len(num_vars, degree, num_queries):
    return N.lib().gb_instance_proof_len(num_vars, degree, num_queries)


class Instance:
    """Host-side instance: polys [degree][2^num_vars] (u64, < p) and its proof buffer."""

    def __init__(self, polys, index, num_queries):
        self.polys = np.ascontiguousarray(np.asarray(polys, dtype=np.uint64))
        self.degree, size = self.polys.shape
        self.num_vars = size.bit_length() - 1
        assert size == 1 << self.num_vars
        self.index = int(index)
        self.num_queries = num_queries
        self.proof = np.zeros(instance_proof_len(self.num_vars, self.degree, num_queries), np.uint64)
        self.device = None

    def to_device(self):
        """Keep the polynomials resident in HBM; later proofs read them from there."""
        from .memory import DeviceBuffer
        if self.device is None:
            self.device = DeviceBuffer.from_numpy(self.polys.reshape(-1))
        return self

    def struct(self):
        if self.device is not None:
            return GbInstance(self.num_vars, self.degree, self.index, None, self.device.ptr, self.proof.ctypes.data)
        return GbInstance(self.num_vars, self.degree, self.index, self.polys.ctypes.data, None,
                          self.proof.ctypes.data)

    def split(self):
        return split_instance_proof(self.proof, self.num_vars, self.degree, self.num_queries)


class MatmulJob:
    """A quantized matmul layer C = A B as a proof job: A [m][k] and B [k][n] int8 (host)."""

    def __init__(self, a, b, index, num_queries):
        self.a = np.ascontiguousarray(np.asarray(a, dtype=np.int8))
        self.b = np.ascontiguousarray(np.asarray(b, dtype=np.int8))
        self.m, self.k = self.a.shape
        k2, self.n = self.b.shape
        assert k2 == self.k
        self.index = int(index)
        self.num_queries = num_queries
        length = N.lib().gb_matmul_proof_len(self.m, self.n, self.k, num_queries)
        if length == 0:
            raise ValueError("m, n, k must be powers of two (k >= 2)")
        self.proof = np.zeros(length, np.uint64)

    def struct(self):
        return GbMatmulJob(self.m, self.n, self.k, self.index, self.a.ctypes.data, self.b.ctypes.data,
                           self.proof.ctypes.data)

    def split(self):
        lm, ln, lk = (self.m.bit_length() - 1, self.n.bit_length() - 1, self.k.bit_length() - 1)
        p, o = self.proof, 0

        def take(k, shape):
            nonlocal o
            v = p[o:o + k].reshape(shape)
            o += k
            return v

        q = self.num_queries
        out = {"roots": take(8, (2, 4)), "claim": take(2, (2,)), "round_messages": take(lk * 6, (lk, 3, 2)),
               "challenges": take(lk * 2, (lk, 2)), "final_evals": take(4, (2, 2)), "final_eval": take(2, (2,))}
        la = N.lib().gb_basefold_proof_len(lm + lk, LOG_RATE, q)
        lb = N.lib().gb_basefold_proof_len(lk + ln, LOG_RATE, q)
        out["open_a"] = take(la, (la,))
        out["open_b"] = take(lb, (lb,))
        out["ajtai"] = take(16 * 64, (16, 64))
        assert o == p.size
        return out


def prove_matmul(table, ajtai_key, master_seed, job):
    """The per-call path for one matmul job."""
    s = job.struct()
    N.check(N.lib().gb_prove_matmul(table.handle, ajtai_key.handle, _seed(master_seed), job.num_queries,
                                    ctypes.byref(s)), "gb_prove_matmul")
    return job.proof


def matmul_stream(count, seed, rate_per_s=200.0, dims=(256, 512, 1024, 4096), num_queries=34):
    """``count`` matmul jobs with M, N, K uniform over ``dims``, int8 values uniform in
    [-128, 127], and Poisson arrival times (seconds from 0) of mean rate ``rate_per_s``."""
    rng = np.random.default_rng(seed)
    arrivals = np.cumsum(rng.exponential(1.0 / rate_per_s, size=count))
    jobs = []
    for k in range(count):
        m, n, kk = (int(x) for x in rng.choice(np.asarray(dims), size=3))
        a = rng.integers(-128, 128, size=(m, kk), dtype=np.int8)
        b = rng.integers(-128, 128, size=(kk, n), dtype=np.int8)
        jobs.append(MatmulJob(a, b, k, num_queries))
    return jobs, arrivals


def split_instance_proof(proof, n, d, q):
    o = 0

    def take(k, shape):
        nonlocal o
        v = proof[o:o + k].reshape(shape)
        o += k
        return v

    roots = take(4 * d, (d, 4))
    msgs = take(n * (d + 1) * 2, (n, d + 1, 2))
    ch = take(2 * n, (n, 2))
    finals = take(2 * d, (d, 2))
    fe = take(2, (2,))
    plen = N.lib().gb_basefold_proof_len(n, LOG_RATE, q)
    opens = [split_proof(take(plen, (plen,)), n, LOG_RATE, q) for _ in range(d)]
    assert o == proof.size
    return {"roots": roots, "round_messages": msgs, "challenges": ch, "final_evals": finals, "final_eval": fe,
            "opens": opens}


def _seed(master_seed):
    return (ctypes.c_uint64 * 2)(int(master_seed[0]), int(master_seed[1]))


def prove_instance(table, master_seed, inst):
    """The per-call path: one instance on the calling thread's stream."""
    s = inst.struct()
    N.check(N.lib().gb_prove_instance(table.handle, _seed(master_seed), inst.num_queries, ctypes.byref(s)),
            "gb_prove_instance")
    return inst.proof


class Schedule:
    """Per-thread scheduling knobs (results never depend on them): the Merkle cooperative threshold
    (gb_set_coop_threshold), the single-CTA top size (gb_set_merkle_top_nodes) and the lockstep
    engine's staggered groups and open parts (gb_set_lockstep_schedule).  A context manager that
    sets the given ones on the calling thread and restores the previous ones."""

    def __init__(self, coop_threshold=None, top_nodes=None, groups=None, open_parts=None):
        self.coop, self.top, self.groups, self.parts = coop_threshold, top_nodes, groups, open_parts

    def __enter__(self):
        L = N.lib()
        g, p = ctypes.c_int(), ctypes.c_int()
        L.gb_get_lockstep_schedule(ctypes.byref(g), ctypes.byref(p))
        self._old = (L.gb_get_coop_threshold(), L.gb_get_merkle_top_nodes(), g.value, p.value)
        if self.coop is not None:
            L.gb_set_coop_threshold(self.coop)
        if self.top is not None:
            L.gb_set_merkle_top_nodes(self.top)
        if self.groups is not None or self.parts is not None:
            N.check(L.gb_set_lockstep_schedule(self.groups if self.groups is not None else g.value,
                                               self.parts if self.parts is not None else p.value),
                    "gb_set_lockstep_schedule")
        return self

    def __exit__(self, *a):
        L = N.lib()
        L.gb_set_coop_threshold(self._old[0])
        L.gb_set_merkle_top_nodes(self._old[1])
        L.gb_set_lockstep_schedule(self._old[2], self._old[3])


def batch_prove(table, master_seed, instances, workers=8, hbm_budget=64 << 30, coop_threshold=None, top_nodes=None,
                engine="service", groups=None, open_parts=None):
    """All instances at once.  engine "service": the prover service, whole instances on worker
    streams, largest first; "lockstep": the round-synchronous engine (commits, sumcheck rounds and
    opening rounds of all instances in lockstep) in `groups` staggered groups whose openings run in
    `open_parts` parts.  The schedule (None keeps the calling thread's) never changes the proofs."""
    if not instances:
        return
    q = instances[0].num_queries
    assert all(i.num_queries == q for i in instances)
    arr = (GbInstance * len(instances))(*[i.struct() for i in instances])
    fn = {"service": N.lib().gb_batch_prove, "lockstep": N.lib().gb_batch_prove_lockstep}[engine]
    with Schedule(coop_threshold, top_nodes, groups, open_parts):
        N.check(fn(table.handle, _seed(master_seed), q, arr, len(instances), workers, hbm_budget),
                "gb_batch_prove" if engine == "service" else "gb_batch_prove_lockstep")


class ProverService:
    """Prover service: submit instances or matmul jobs as they arrive; each is admitted as soon as
    its estimated device footprint fits the HBM budget beside the jobs in flight.

    continuous=False: a worker proves a job whole on its own stream (gb_prover_create).
    continuous=True: workers run each job's steps before its openings, then its openings join the
    service's open engines, which advance every opening in flight one round per step with one
    launch per kernel kind for all of them (gb_prover_create_continuous)."""

    def __init__(self, table, master_seed, num_queries, workers=8, hbm_budget=64 << 30, coop_threshold=None,
                 top_nodes=None, continuous=False, slots=None):
        self.handle = ctypes.c_void_p()
        self.num_queries = num_queries
        fn = "gb_prover_create_continuous" if continuous else "gb_prover_create"
        N.check(getattr(N.lib(), fn)(table.handle, _seed(master_seed), num_queries, workers, hbm_budget,
                                     ctypes.byref(self.handle)), fn)
        if slots is not None:
            N.check(N.lib().gb_prover_set_slots(self.handle, slots), "gb_prover_set_slots")
        if coop_threshold is not None:
            N.check(N.lib().gb_prover_set_coop_threshold(self.handle, coop_threshold), "gb_prover_set_coop_threshold")
        if top_nodes is not None:
            N.check(N.lib().gb_prover_set_merkle_top_nodes(self.handle, top_nodes), "gb_prover_set_merkle_top_nodes")
        self._live = {}

    def set_ajtai_key(self, key):
        """Key for matmul jobs (an AjtaiKey of 16 rows over 1024 ring columns)."""
        self._key = key
        N.check(N.lib().gb_prover_set_ajtai_key(self.handle, key.handle), "gb_prover_set_ajtai_key")

    def submit(self, job):
        """Submit an Instance or a MatmulJob; returns its ticket."""
        assert job.num_queries == self.num_queries
        s = job.struct()
        t = ctypes.c_uint64()
        if isinstance(job, MatmulJob):
            N.check(N.lib().gb_prover_submit_matmul(self.handle, ctypes.byref(s), ctypes.byref(t)),
                    "gb_prover_submit_matmul")
        else:
            N.check(N.lib().gb_prover_submit(self.handle, ctypes.byref(s), ctypes.byref(t)), "gb_prover_submit")
        self._live[t.value] = job  # keeps the host buffers alive until waited for
        return t.value

    def running(self):
        """Jobs admitted and not yet complete."""
        return int(N.lib().gb_prover_running(self.handle))

    def openings_in_flight(self):
        """Openings in the continuous service's open engines (0 for the whole-job service)."""
        return int(N.lib().gb_prover_openings_in_flight(self.handle))

    def wait(self, ticket):
        st = GbJobStats()
        rc = N.lib().gb_prover_wait(self.handle, ticket, ctypes.byref(st))
        inst = self._live.pop(ticket, None)
        N.check(rc, "gb_prover_wait")
        return inst, {"queued_ms": st.queued_ms, "run_ms": st.run_ms, "latency_ms": st.latency_ms}

    def close(self):
        if self.handle:
            N.lib().gb_prover_drain(self.handle)
            N.lib().gb_prover_destroy(self.handle)
            self.handle = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def mixed_workload(count, seed, min_vars=10, max_vars=20, degrees=(2, 3, 4), num_queries=34):
    """``count`` instances with log2 size uniform over the integers [min_vars, max_vars] and
    degree uniform over ``degrees``; values uniform in [0, p) from a seeded generator."""
    rng = np.random.default_rng(seed)
    sizes = rng.integers(min_vars, max_vars + 1, size=count)
    degs = rng.choice(np.asarray(degrees), size=count)
    out = []
    for k in range(count):
        polys = rng.integers(0, P, size=(int(degs[k]), 1 << int(sizes[k])), dtype=np.uint64)
        out.append(Instance(polys, k, num_queries))
    return out


def autotune_lockstep(table, master_seed, instances, groups=(2, 1, 3, 4), open_parts=(2, 1, 3),
                      coop_thresholds=(16384, 8192, 32768), hbm_budget=64 << 30, repeats=1):
    """Schedule (groups, open parts, cooperative threshold) of the lockstep engine for this batch,
    by coordinate search in that order from the first value of each axis, each candidate timed
    by wall clock (the best of `repeats` runs) after one warm-up run.  Returns
    ((groups, open_parts, coop), {schedule: seconds})."""
    def run(g, p, c):
        best_t = None
        for _ in range(repeats):
            t0 = time.perf_counter()
            batch_prove(table, master_seed, instances, 1, hbm_budget, coop_threshold=c, engine="lockstep",
                        groups=g, open_parts=p)
            t = time.perf_counter() - t0
            best_t = t if best_t is None else min(best_t, t)
        return best_t

    best = (groups[0], open_parts[0], coop_thresholds[0])
    run(*best)
    times = {}
    for axis, values in ((0, groups), (1, open_parts), (2, coop_thresholds)):
        for v in values:
            cand = list(best)
            cand[axis] = v
            cand = tuple(cand)
            if cand not in times:
                times[cand] = run(*cand)
        best = min(times, key=times.get)
    return best, times


def autotune(table, master_seed, instances, workers=(8, 12, 16, 24), coop_thresholds=(16384, 4096),
             top_nodes=(16, 256, 2048), hbm_budget=64 << 30):
    """Schedule (workers, cooperative threshold, top size) for this batch by coordinate search:
    after a warm-up run, the worker count at the default Merkle schedule, then the
    cooperative threshold, then the top size, each measured by wall time.  Few concurrent
    proofs favour latency (8-lane permutations, small single-CTA tops); many favour throughput
    and fewer launches.  Returns ((workers, coop, top), {schedule: seconds})."""
    def run(w, c, t):
        t0 = time.perf_counter()
        batch_prove(table, master_seed, instances, w, hbm_budget, coop_threshold=c, top_nodes=t)
        return time.perf_counter() - t0

    best = (workers[0], coop_thresholds[0], top_nodes[0])
    run(*best)
    times = {}
    for axis, values in ((0, workers), (1, coop_thresholds), (2, top_nodes)):
        for v in values:
            cand = list(best)
            cand[axis] = v
            cand = tuple(cand)
            if cand not in times:
                times[cand] = run(*cand)
        best = min(times, key=times.get)
    return best, times
