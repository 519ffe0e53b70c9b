"""Benchmark: Basefold commit + open_ext2 proofs on one GB300 (proofs/sec).

Workload (the reference's Basefold configuration): one multilinear polynomial of
2^22 Goldilocks evaluations uniform in [0, p) from a fixed seed, rate 1/2
(codeword 2^23), Poseidon2-w8 Merkle trees, 22 fold rounds with the interleaved
sumcheck, 34 queries (the reference key's default), folding table
BasefoldTable::generate(22, 1, 22, seed 42) resident on the device.  One step =
commit + open of one proof with a fresh per-proof transcript.

value: steps with evaluations already in HBM (device-timed with CUDA events on the
       library's launch stream, L2 flushed between steps).
e2e:   the same step through the C ABI from pinned host evaluations (host->device
       copy inside the timed region) with the proof returned to host memory.

--impl reference runs the CPU restatement of the reference's prover (the
reference is Rust; its toolchain is absent) on a bounded sample and prints the
same JSON line with impl=reference.
"""
import argparse
import ctypes
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

P = 0xFFFFFFFF00000001
N_VARS, LOG_RATE, QUERIES, TABLE_SEED = 22, 1, 34, 42
METRIC = "proofs/sec"


def env_rank():
    return int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1"))


def max_over_ranks(values, dist, device):
    """Each value's maximum over the ranks (the slowest rank's time), through the default process
    group when dist (nccl on the GPUs, gloo in the CPU tests)."""
    import torch
    t = torch.tensor([float(v) for v in values], dtype=torch.float64, device=device)
    if dist:
        import torch.distributed as tdist
        tdist.all_reduce(t, op=tdist.ReduceOp.MAX)
    return [float(v) for v in t.tolist()]


def replica_throughput(world, ms_max):
    """Proofs per second of world replicas that each prove one proof per step of ms_max."""
    return world * 1000.0 / ms_max


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    def __init__(self):
        self.samples = []
        self._stop = threading.Event()
        self._th = None

    def _run(self):
        q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
             "clocks_event_reasons.sw_power_cap")
        while not self._stop.is_set():
            try:
                out = subprocess.run(["nvidia-smi", f"--query-gpu={q}", "--format=csv,noheader,nounits", "-i", "0"],
                                     capture_output=True, text=True, timeout=5).stdout.strip()
                if out:
                    self.samples.append([x.strip() for x in out.splitlines()[0].split(",")])
            except Exception:
                pass
            self._stop.wait(0.2)

    def __enter__(self):
        self._th = threading.Thread(target=self._run, daemon=True)
        self._th.start()
        return self

    def __exit__(self, *a):
        self._stop.set()
        self._th.join(timeout=10)

    def summary(self):
        if not self.samples:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(s[0]) for s in self.samples if s[0].replace(".", "").isdigit()]
        mx = [float(s[1]) for s in self.samples if s[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for s in self.samples for i in range(4) if len(s) > 3 + i and s[3 + i] == "Active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.samples)}


def measured_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return d.get("hbm_gbs", 6800.0), "measured"
    except Exception:
        return 6800.0, "fallback"


def cpu_basefold_proofs(steps, warmup, n=N_VARS, seed=1234):
    """Commit + open_ext2 proofs of 2^n evaluations by the C restatement of the reference's CPU
    prover (cpu_full_open_ext2, zk-torch-3/src/commit/cpu_basefold.rs:235-425), each proof's large
    loops (Merkle layers, transform layers, folds, sums) split over every host thread.  The folding
    table is the key's, generated once outside the timed proofs, as BasefoldTable::generate is.
    Returns the seconds of each timed proof, the thread count and the last proof."""
    import oracle as O
    O.build(ref_root="")
    threads = os.cpu_count() or 1
    O.set_threads(threads)
    rng = np.random.default_rng(seed)
    ev = rng.integers(0, P, size=1 << n, dtype=np.uint64)
    pt = rng.integers(0, P, size=(n, 2), dtype=np.uint64)
    table = O.basefold_table(n, LOG_RATE, n, TABLE_SEED)

    def one():
        c = O.basefold_commit(ev, LOG_RATE)
        return c, O.basefold_open_ext2(c, pt, table, O.Transcript(b"bf-open"), QUERIES)
    for _ in range(warmup):
        one()
    secs, last = [], None
    for _ in range(steps):
        t0 = time.perf_counter()
        last = one()
        secs.append(time.perf_counter() - t0)
    return secs, threads, last


def run_reference(args):
    """The reference's CPU prover path, restated in C (the reference is Rust and no Rust
    toolchain exists here or on the GPU machine), at the full 2^22 configuration on all host
    threads: each step is one real commit + open_ext2 proof.  Rank 0 only."""
    rank, world = env_rank()
    if rank != 0:
        return
    warm = min(args.warmup, 1)  # a CPU proof has no device state to warm; one untimed proof
    secs, threads, _ = cpu_basefold_proofs(args.steps, warm)
    step_s = statistics.mean(secs)
    value = 1.0 / step_s
    sample = (f"{args.steps} timed commit+open_ext2 proofs of 2^{N_VARS} evaluations (C restatement), "
              f"each split over {threads} host threads, after {warm} untimed proof; table generated once")
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "proofs/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": warm, "warmup_requested": args.warmup, "ms_per_step": step_s * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u64 (Goldilocks)",
        "data": "synthetic",
        "config": {"workload": f"basefold commit+open_ext2, 2^{N_VARS} evals, rate 1/2, {QUERIES} queries",
                   "num_vars": N_VARS, "log_rate": LOG_RATE, "num_queries": QUERIES, "table_seed": TABLE_SEED},
        "cpu_baseline": {"value": value, "unit": "proofs/s", "cores": threads, "kind": "port", "sample": sample},
        "e2e": {"value": value, "unit": "proofs/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "step_ms_all": [round(t * 1e3, 1) for t in secs],
    }
    print(json.dumps(line))


def cpu_baseline_sample(gpu_proof=None, seed=1234):
    """One full-size CPU proof (after a small untimed one), on all host threads; the proof is
    compared with the GPU's proof of the same inputs when one is given."""
    cpu_basefold_proofs(0, 1, n=14)
    secs, threads, (_, proof) = cpu_basefold_proofs(1, 0, seed=seed)
    out = {"value": 1.0 / secs[0], "unit": "proofs/s", "cores": threads, "kind": "port",
           "sample": f"1 commit+open_ext2 proof of 2^{N_VARS} evaluations (C restatement) split over {threads} "
                     f"host threads, {secs[0]:.1f} s; table generated once, outside the timing"}
    if gpu_proof is not None:
        out["identical_to_gpu_proof"] = bool(np.array_equal(np.asarray(gpu_proof), proof))
    return out


def cpu_sumcheck_sample(polys, gpu_msgs=None, reps=3):
    """CpuLinearSumcheckProverExt2 (zk-torch-3/src/sumcheck/cpu_ext2_prover.rs:13-110), single-threaded
    like the reference's, restated in C: 2 x 2^20, whole proof with its transcript."""
    import oracle as O
    O.set_threads(1)
    secs = []
    for _ in range(reps):
        t0 = time.perf_counter()
        ref = O.sumcheck_prove_ext2(O.Transcript(b"bench"), polys)
        secs.append(time.perf_counter() - t0)
    s = statistics.median(secs)
    out = {"value": polys.size / s / 1e6, "unit": "Melem/s", "cores": 1, "kind": "port",
           "sample": f"{reps} Ext2-challenge sumcheck proofs of 2 x 2^20 (C restatement, one thread as the "
                     f"reference's CpuLinearSumcheckProverExt2), median {s * 1e3:.0f} ms"}
    if gpu_msgs is not None:
        out["identical_to_gpu_proof"] = bool(np.array_equal(np.asarray(gpu_msgs), ref["round_messages"]))
    return out


def cpu_ajtai_sample(key, z8, rows, gpu_out=None):
    """The Ajtai commitment by the C restatement (ajtai_cpu_reference.cuh:57-186 semantics, exact
    128-bit accumulation), witnesses split over every host thread."""
    import oracle as O
    threads = os.cpu_count() or 1
    O.set_threads(threads)
    t0 = time.perf_counter()
    ref = O.ajtai_commit_u8_batch(key, z8, 0, rows)
    s = time.perf_counter() - t0
    out = {"value": z8.shape[0] / s, "unit": "commitments/s", "cores": threads, "kind": "port",
           "sample": f"{z8.shape[0]} witnesses x {z8.shape[1]} coefficients, rows 0..{rows - 1} (C restatement, "
                     f"witnesses over {threads} host threads, matrix generation included), {s:.2f} s"}
    if gpu_out is not None:
        out["identical_to_gpu"] = bool(np.array_equal(np.asarray(gpu_out).reshape(ref.shape), ref))
    return out


def batch_open_cpu_sample(num_claims, sample_vars=12, n=20):
    """The C restatement of batch_open_ext2 (one core) on 8 polys x 2^sample_vars at 2 points,
    time scaled by 2^(n - sample_vars) to the 2^n workload."""
    import oracle as O
    O.build(ref_root="")
    rng = np.random.default_rng(7)
    comms = [O.basefold_commit(rng.integers(0, P, size=1 << sample_vars, dtype=np.uint64), LOG_RATE) for _ in range(8)]
    points = [rng.integers(0, P, size=(sample_vars, 2), dtype=np.uint64) for _ in range(2)]
    claims = [(j, k, rng.integers(0, P, size=2, dtype=np.uint64)) for j in range(8) for k in range(2)]
    table = O.basefold_table(sample_vars, LOG_RATE, sample_vars, TABLE_SEED)
    t0 = time.perf_counter()
    O.basefold_batch_open_ext2(comms, points, claims, table, O.Transcript(b"bf-batch"), QUERIES)
    wall = (time.perf_counter() - t0) * (1 << (n - sample_vars))
    return {"value": num_claims / wall, "unit": "claims/s", "cores": 1, "kind": "port",
            "sample": f"one batch opening of 8 polys x 2^{sample_vars} at 2 points (C restatement, one core), "
                      f"time scaled x{1 << (n - sample_vars)} to 2^{n}"}


def run_side_workload(args):
    """Configs other than the headline, each on one GPU with inputs resident in HBM."""
    import torch
    from morpheus_gb300 import build as B
    B.build()
    from morpheus_gb300 import _native as Nn
    from morpheus_gb300.memory import DeviceBuffer
    L = Nn.lib()
    stream = torch.cuda.Stream()
    L.gb_set_stream(ctypes.c_void_p(stream.cuda_stream))
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")
    rng = np.random.default_rng(99)

    def ev_time(fn):
        with torch.cuda.stream(stream):
            flush.zero_()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        fn()
        e1.record(stream)
        e1.synchronize()
        return e0.elapsed_time(e1)

    if args.workload == "sumcheck":
        from morpheus_gb300.sumcheck import GpuLinearSumcheckProver, Transcript
        n, d = 20, 2
        polys = DeviceBuffer.from_numpy(rng.integers(0, P, size=d << n, dtype=np.uint64))

        def step():
            t = Transcript(b"bench")
            GpuLinearSumcheckProver(n, d, t).prove((polys, d), t)
        unit, metric, work = "Melem/s", "sumcheck Melem/s", d * (1 << n) / 1e6
        cfg = {"workload": "product sumcheck, 2 polys x 2^20 Goldilocks, Ext2 challenges, 20 rounds"}
    elif args.workload == "batch_open":
        from morpheus_gb300.basefold import BasefoldCommitment, BasefoldTable, batch_open_ext2
        from morpheus_gb300.sumcheck import Transcript
        n, npoly, npts, q = 20, 8, 2, QUERIES
        tab = BasefoldTable.generate(n, LOG_RATE, n, TABLE_SEED)
        comms = [BasefoldCommitment.commit(rng.integers(0, P, size=1 << n, dtype=np.uint64), n, LOG_RATE)
                 for _ in range(npoly)]
        points = [rng.integers(0, P, size=(n, 2), dtype=np.uint64) for _ in range(npts)]
        claims = [(j, k, rng.integers(0, P, size=2, dtype=np.uint64)) for j in range(npoly) for k in range(npts)]

        def step():
            t = Transcript(b"bf-batch")
            batch_open_ext2(comms, points, claims, tab, t, q)
        unit, metric, work = "claims/s", "batch_open_ext2 claims/s", float(len(claims))
        cfg = {"workload": f"batch_open_ext2: {npoly} polys x 2^{n}, {npts} points, {len(claims)} claims, "
                           f"rate 1/2, {q} queries", "l2": "flushed between timed steps"}
    elif args.workload == "peval":
        from morpheus_gb300 import partial_eval as PE
        n, m = 26, 14  # einsum A input 2^14 x 2^12, its halves swapped, the 2^14 side summed
        ranges = [(12, 26), (0, 12)]
        half = n // 2
        lo, hi = PE.build_split_luts(n, ranges, half)
        d_ev = DeviceBuffer.from_numpy(rng.integers(0, P, size=1 << n, dtype=np.uint64))
        d_lo, d_hi = DeviceBuffer.from_numpy(lo), DeviceBuffer.from_numpy(hi)
        d_eq, keep = PE.eq_table_ext2_device(rng.integers(0, P, size=(m, 2), dtype=np.uint64))
        d_out = DeviceBuffer(2 << (n - m))

        def step():
            Nn.check(L.fused_permute_partial_eval_ffi(d_ev.ptr, d_out.ptr, d_eq.ptr, d_lo.ptr, d_hi.ptr, n, m, half,
                                                      1 << (n - m), 0), "fused")
        unit, metric = "GB/s", "fused permute + partial eval GB/s"
        work = ((1 << n) * 8 + (1 << m) * 16 + (2 << (n - m)) * 8) / 1e9
        cfg = {"workload": f"fused_permute_partial_eval: 2^{n} evaluations (2^14 x 2^12 einsum input, halves "
                           f"swapped), {m} variables fixed at Ext2 challenges", "l2": "flushed between timed steps"}
    elif args.workload == "fold":
        nf = 24
        src_buf = DeviceBuffer.from_numpy(rng.integers(0, P, size=2 * 2 * (1 << nf), dtype=np.uint64))
        dst_buf = DeviceBuffer(2 * 2 * (1 << (nf - 1)))
        msg = DeviceBuffer(16)
        work_buf = DeviceBuffer.from_numpy(np.zeros(L.gb_sumcheck_round_workspace_words(), np.uint64))

        def step():
            Nn.check(L.gb_sumcheck_fold_round_ext2(src_buf.ptr, 0, 1 << nf, dst_buf.ptr, 1 << (nf - 1), 2,
                                                   1 << (nf - 2), 5, 7, msg.ptr, work_buf.ptr), "fold round")
        unit, metric = "GB/s", "fused fold round GB/s"
        work = (2 * (1 << nf) * 16 + 2 * (1 << (nf - 1)) * 16) / 1e9
        cfg = {"workload": "sumcheck fold round: 2 polys x 2^24 Ext2 folded with an Ext2 challenge to 2 x 2^23, "
                           "next round's degree-2 message", "l2": "flushed between timed launches"}
    else:
        n_ring, Bw, rows = 1024, args.witnesses, 16
        key = np.array([0x5EED, 1, 2, 3, 4, 5, 6, 7], np.uint32)
        h = ctypes.c_void_p()
        Nn.check(L.gb_ajtai_key_create(key.ctypes.data, 0, rows, n_ring, ctypes.byref(h)), "key")
        L.gb_ajtai_set_batch_form(args.ajtai_form)
        z = DeviceBuffer.from_numpy(rng.integers(0, 256, size=Bw * n_ring * 64, dtype=np.uint8))
        out = DeviceBuffer(Bw * rows * 64)

        def step():
            Nn.check(L.gb_ajtai_commit_u8_batched(h, z.ptr, Bw, out.ptr), "ajtai")
        unit, metric, work = "commitments/s", "ajtai witness commitments/s", float(Bw)
        cfg = {"workload": f"ajtai commit, {Bw} witnesses x 2^16 coefficients in [0,256), rows 0..15, "
                           "q = 2^64-2^32-31", "form": ["by batch size", "witness-circulant", "key-Toeplitz",
                                                                "key-Toeplitz on CTA pairs",
                                                                "Hankel key windows on CTA pairs"][args.ajtai_form],
               "l2": "flushed between timed steps"}
    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    times = [ev_time(step) for _ in range(args.steps)]
    ms = statistics.mean(times)
    line = {"metric": metric, "value": work / (ms * 1e-3), "unit": unit, "n_gpus": 1, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "bf16 limbs (exact), u64 out" if args.workload == "ajtai" else "u64",
            "data": "synthetic", "config": cfg, "step_ms_all": [round(t, 4) for t in times]}
    if args.workload == "batch_open":
        line["cpu_baseline"] = batch_open_cpu_sample(len(claims))
    if args.workload == "peval":
        # the unfused path on the same evaluations (no permutation): partial_eval_ext2_from_gl
        d_r = DeviceBuffer.from_numpy(rng.integers(0, P, size=2 * m, dtype=np.uint64))
        d_half = DeviceBuffer(2 << (n - 1))
        pe = lambda: Nn.check(L.partial_eval_ext2_from_gl_ffi(d_ev.ptr, d_half.ptr, d_r.ptr, n, m), "peval")
        pe()
        pe_ms = min(ev_time(pe) for _ in range(5))
        pe_bytes = (1 << n) * 8 + (2 << (n - 4)) * 8 * 2  # first pass reads 2^n, writes 2^(n-4) Ext2
        line["partial_eval_ext2"] = {"ms": pe_ms, "GB_s": pe_bytes / (pe_ms * 1e-3) / 1e9,
                                     "workload": f"partial_eval_ext2_from_gl_ffi, 2^{n} evaluations, {m} variables"}
    if args.workload in ("fold", "peval"):
        peak, src = measured_peaks()
        line["roofline"] = {"bound": "hbm", "achieved": line["value"], "peak": peak, "unit": "GB/s",
                            "frac": line["value"] / peak, "peak_source": src}
    if args.workload == "ajtai":
        line["tensor_tflops_equiv"] = 2.0 * 8 * rows * 64 * Bw * n_ring * 64 / (ms * 1e-3) / 1e12
        # whole batch (digit prep, GEMM, combine) against the tensor bound (the Hankel form) or the
        # HBM bound of the GEMM's operand stream (the other forms)
        peak, src = measured_peaks()
        circulant = args.ajtai_form == 1 or (args.ajtai_form == 0 and Bw <= 104)
        hankel = args.ajtai_form == 4 or (args.ajtai_form == 0 and Bw > 104)
        pair = args.ajtai_form == 3
        if circulant:  # the key's digit planes once (16 MB) plus the witness bytes
            op_bytes = 8 * rows * n_ring * 64 * 2 + Bw * n_ring * 64
        elif hankel:  # the key's Hankel windows once (3840 B per 128 rows and ring column) plus the witness digits
            op_bytes = 4 * rows * n_ring * 3840 + Bw * n_ring * 64 * 2
        else:  # the key's Toeplitz expansion once (1.07 GB) plus the witness digits
            op_bytes = 8 * rows * 64 * n_ring * 64 * 2 + Bw * n_ring * 64 * 2
        try:
            with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
                tpeak = json.load(f).get("bf16_tflops", 1900.0)
        except Exception:
            tpeak = 1900.0
        kernel = ("ajtai_gemm_wc_kernel" if circulant else
                  "ajtai_gemm_pair_kernel<true> (Hankel windows)" if hankel else
                  "ajtai_gemm_pair_kernel<false>" if pair else "ajtai_gemm_kernel") + " (whole batch timed)"
        hbm = {"achieved_GB_s": op_bytes / (ms * 1e-3) / 1e9, "peak_GB_s": peak, "peak_source": src,
               "bytes_per_launch": op_bytes}
        if hankel:  # reads a quarter of the expansion's bytes and keeps the tensor pipe busy: tensor-bound
            line["roofline"] = {"bound": "tensor", "kernel": kernel, "achieved": line["tensor_tflops_equiv"],
                                "peak": tpeak, "unit": "TFLOP/s", "frac": line["tensor_tflops_equiv"] / tpeak,
                                "peak_source": "measured (bf16 burst)", "hbm": hbm, "traffic": None}
        else:
            line["roofline"] = {"bound": "hbm", "kernel": kernel, "achieved": hbm["achieved_GB_s"], "peak": peak,
                                "unit": "GB/s", "frac": hbm["achieved_GB_s"] / peak, "peak_source": src,
                                "bytes_per_launch": op_bytes, "tensor_frac": line["tensor_tflops_equiv"] / tpeak,
                                "traffic": None}
        # the fold tree at the SuperNeo shape: 50 binary + 13 ternary witnesses of 2^14 ring elements
        nb, nt, nr = 50, 13, 1 << 14
        zb = DeviceBuffer.from_numpy(rng.integers(0, 2**63, size=nb * nr, dtype=np.uint64))
        pn = rng.integers(0, 2**63, size=(2, nt * nr), dtype=np.uint64)
        d_pos, d_neg = DeviceBuffer.from_numpy(pn[0]), DeviceBuffer.from_numpy(pn[1] & ~pn[0])
        r = rng.choice(np.array([-1, 0, 1, 2], np.int8), size=(nb + nt) * 64)
        d_r = DeviceBuffer.from_numpy(r)
        d_o = DeviceBuffer(nr * 64, np.int16)
        mf = lambda: Nn.check(L.ajtai_multifold_mixed_witness_ffi(zb.ptr, d_pos.ptr, d_neg.ptr, d_r.ptr, d_o.ptr, nb, nt,
                                                                   nr, 256), "multifold")
        mf()
        mf_ms = min(ev_time(mf) for _ in range(5))
        line["multifold_mixed"] = {"ms": mf_ms, "workload": f"{nb} binary + {nt} ternary witnesses x {nr} ring "
                                                             "elements, challenges in {-1, 0, 1, 2}"}
    print(json.dumps(line))


def ajtai_c3_summary(L, Nn, DeviceBuffer, ev_time):  # ev_time flushes L2 before it times
    """Compact line for the Ajtai configuration: the whole 256-witness batch (digit prep, tensor-core
    GEMM, combine), its tensor and HBM rooflines, and the C restatement on the host cores; beside
    it one witness alone (the served jobs' commitment) in both GEMM forms.  L2 flushed before
    every timed call."""
    n_ring, Bw, rows = 1024, 256, 16
    key = np.array([0x5EED, 1, 2, 3, 4, 5, 6, 7], np.uint32)
    z_host = np.random.default_rng(303).integers(0, 256, size=(Bw, n_ring * 64), dtype=np.uint8)
    h = ctypes.c_void_p()
    Nn.check(L.gb_ajtai_key_create(key.ctypes.data, 0, rows, n_ring, ctypes.byref(h)), "ajtai key")
    z = DeviceBuffer.from_numpy(z_host.reshape(-1))
    out = DeviceBuffer(Bw * rows * 64)
    timed = ev_time  # flushes L2 on the launch stream, then times
    step = lambda: Nn.check(L.gb_ajtai_commit_u8_batched(h, z.ptr, Bw, out.ptr), "ajtai")
    for _ in range(3):
        step()
    times = [timed(step) for _ in range(10)]
    ms = statistics.median(times)
    got = out.to_numpy()
    # the same batch through the key's Toeplitz expansion (1.07 GB), on one CTA per SM and on CTA
    # pairs; the automatic choice reads the Hankel windows (252 MB) on CTA pairs
    other = {}
    for name, form in (("one_cta_toeplitz", 2), ("pair_toeplitz", 3)):
        old = L.gb_ajtai_set_batch_form(form)
        for _ in range(2):
            step()
        other[name] = statistics.median(timed(step) for _ in range(10))
        assert np.array_equal(out.to_numpy(), got)
        L.gb_ajtai_set_batch_form(old)
    # one witness: the automatic form (witness-circulant) against the key-Toeplitz form
    one = {}
    for name, form in (("auto", 0), ("toeplitz", 2)):
        old = L.gb_ajtai_set_batch_form(form)
        step1 = lambda: Nn.check(L.gb_ajtai_commit_u8_batched(h, z.ptr, 1, out.ptr), "ajtai one")
        for _ in range(3):
            step1()
        one[name] = statistics.median(timed(step1) for _ in range(10))
        one[name + "_out"] = out.to_numpy()[:rows * 64].copy()
        L.gb_ajtai_set_batch_form(old)
    assert np.array_equal(one["auto_out"], one["toeplitz_out"]) and np.array_equal(one["auto_out"], got[:rows * 64])
    Nn.check(L.gb_ajtai_key_destroy(h), "ajtai key destroy")
    peaks = {}
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            peaks = json.load(f)
    except Exception:
        pass
    tpeak = peaks.get("bf16_tflops", 1900.0)
    hpeak = peaks.get("hbm_gbs", 6800.0)
    flop = 2.0 * 8 * rows * 64 * Bw * n_ring * 64  # 8 digit planes of the 1024 x 65536 x 256 product
    alg_bytes = Bw * n_ring * 64 + rows * n_ring * 64 * 8 + Bw * rows * 64 * 8  # Z (u8) + M + out
    tf = flop / (ms * 1e-3) / 1e12
    return {"ms_per_batch": ms, "value": Bw / (ms * 1e-3), "unit": "commitments/s",
            "form": "CTA-pair GEMM on the key's Hankel windows (ajtai_gemm_pair_kernel<true>)",
            "ms_other_forms": other,
            "roofline": {"bound": "tensor", "achieved": tf, "peak": tpeak, "unit": "TFLOP/s", "frac": tf / tpeak,
                         "peak_source": "measured (bf16 burst)" if peaks else "fallback",
                         "hbm_algorithmic_GB_s": alg_bytes / (ms * 1e-3) / 1e9, "hbm_peak": hpeak,
                         "algorithmic_bytes": alg_bytes},
            "single_witness": {"ms_witness_circulant": one["auto"], "ms_key_toeplitz": one["toeplitz"],
                               "identical": True, "note": "one 2^16-coefficient witness, as in a served job; "
                                                         "the automatic choice takes the witness-circulant "
                                                         "form up to 104 witnesses"},
            "cpu_baseline": cpu_ajtai_sample(key, z_host[:64], rows, got.reshape(Bw, rows, 64)[:64]),
            "step_ms_all": [round(t, 4) for t in times],
            "workload": "256 witnesses x 2^16 coefficients in [0, 256), rows 0..15 of the ChaCha8 matrix, "
                        "q = 2^64 - 2^32 - 31; python bench.py --workload ajtai for the full line"}


def run_batched(args, summary=False):
    """Mixed batch of independent instances (product sumcheck + Basefold commit/open of every
    polynomial at the sumcheck point): the prover service with an autotuned worker count
    against the per-call path (the same instances one after another on one stream)."""
    import torch
    from morpheus_gb300 import build as B
    B.build()
    from morpheus_gb300 import _native as Nn
    from morpheus_gb300 import batch
    from morpheus_gb300.basefold import BasefoldTable
    L = Nn.lib()
    count = args.instances
    seed = (0x243F6A8885A308D3 % P, 0x13198A2E03707344 % P)
    table = BasefoldTable.generate(N_VARS, LOG_RATE, N_VARS, TABLE_SEED)
    insts = batch.mixed_workload(count, seed=2026, min_vars=10, max_vars=20, degrees=(2, 3, 4), num_queries=QUERIES)
    elems = sum(i.degree << i.num_vars for i in insts)
    for i in insts:
        i.to_device()
    torch.cuda.synchronize()

    def wall(fn):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        fn()
        torch.cuda.synchronize()
        return time.perf_counter() - t0

    if getattr(args, "quick", False):
        # the lockstep engine alone at the schedule its autotuner settles on for this batch
        # (3 staggered groups, 2 open parts, cooperative threshold 4096), for profiling captures
        with batch.Schedule(4096, None, 3, 2):
            for _ in range(args.warmup):
                batch.batch_prove(table, seed, insts, 16, 160 << 30, engine="lockstep")
            l0 = L.gb_launch_count()
            times = [wall(lambda: batch.batch_prove(table, seed, insts, 16, 160 << 30, engine="lockstep"))
                     for _ in range(args.steps)]
            launches = (L.gb_launch_count() - l0) // max(1, args.steps)
            phase = (ctypes.c_double(), ctypes.c_double(), ctypes.c_double())
            L.gb_lockstep_last_timing(*(ctypes.byref(x) for x in phase))
        print(json.dumps({"metric": "proofs/sec (mixed batch, lockstep only)", "value": count / statistics.mean(times),
                          "unit": "proofs/s", "instances": count, "ms_per_step": statistics.mean(times) * 1e3,
                          "gpu_launches": int(launches),
                          "commit_sumcheck_ms": phase[0].value, "open_ms": phase[1].value,
                          "sumcheck_ms": phase[2].value}))
        return
    # per-call path: a few warm-up instances, then every instance alone, in order
    for i in insts[:8]:
        batch.prove_instance(table, seed, i)

    def per_call():
        for i in insts:
            batch.prove_instance(table, seed, i)
    per_call_s = min(wall(per_call) for _ in range(max(1, args.per_call_steps)))
    alone = [i.proof.copy() for i in insts]

    # batched: tune the schedule on this batch (these runs are the warm-up), then time; the
    # summary mode takes the schedule the full run settles on
    if summary:
        (best, coop, top), tune = (16, 4096, 16), {}
    else:
        (best, coop, top), tune = batch.autotune(table, seed, insts)
    L.gb_set_coop_threshold(coop)
    L.gb_set_merkle_top_nodes(top)
    for _ in range(0 if summary else max(0, args.warmup - 1)):
        batch.batch_prove(table, seed, insts, best)
    same = 0
    if not summary:
        l0 = L.gb_launch_count()
        with ClockSampler() as clk_svc:
            times_svc = [wall(lambda: batch.batch_prove(table, seed, insts, best)) for _ in range(args.steps)]
        launches_svc = (L.gb_launch_count() - l0) // max(1, args.steps)
        same = sum(np.array_equal(i.proof, a) for i, a in zip(insts, alone))
    # the round-synchronous engine on the same batch (same worker count for commits + sumchecks)
    for i in insts:
        i.proof[:] = 0
    if summary:
        times_svc, launches_svc, clk_svc = [float("inf")], 0, None
    budget = 160 << 30
    # the lockstep engine's schedule (staggered groups, open parts, cooperative threshold), tuned
    # on this batch; these runs are its warm-up
    (ls_groups, ls_parts, ls_coop), tune_ls = batch.autotune_lockstep(
        table, seed, insts, groups=(2, 1, 3, 4), open_parts=(2, 1, 3), coop_thresholds=(4096, 16384, 8192, 2048),
        hbm_budget=budget)
    ls_sched = batch.Schedule(ls_coop, None, ls_groups, ls_parts)
    with ls_sched:
        batch.batch_prove(table, seed, insts, best, budget, engine="lockstep")
        l1 = L.gb_launch_count()
        with ClockSampler() as clk_ls:
            times_ls = [wall(lambda: batch.batch_prove(table, seed, insts, best, budget, engine="lockstep"))
                        for _ in range(args.steps)]
        launches_ls = (L.gb_launch_count() - l1) // max(1, args.steps)
        phase = (ctypes.c_double(), ctypes.c_double(), ctypes.c_double())
        L.gb_lockstep_last_timing(*(ctypes.byref(x) for x in phase))
    lockstep_schedule = {"groups": ls_groups, "open_parts": ls_parts, "coop_threshold": ls_coop,
                         "autotune_s": {f"{k[0]}g/{k[1]}p/{k[2]}": round(v, 4) for k, v in tune_ls.items()}}
    same_ls = sum(np.array_equal(i.proof, a) for i, a in zip(insts, alone))
    engine = "lockstep" if statistics.mean(times_ls) < statistics.mean(times_svc) else "service"
    times, launches, clk = (times_ls, launches_ls, clk_ls) if engine == "lockstep" else (times_svc, launches_svc, clk_svc)
    if summary:
        return {"value": count / statistics.mean(times), "unit": "proofs/s", "instances": count,
                "engine": engine, "ms_per_batch": statistics.mean(times) * 1e3,
                "per_call": {"value": count / per_call_s, "unit": "proofs/s", "ms_per_batch": per_call_s * 1e3},
                "batched_over_per_call": per_call_s / statistics.mean(times),
                "identical_to_per_call": f"{same_ls}/{count}", "gpu_launches": int(launches),
                "lockstep_schedule": lockstep_schedule,
                "workload": "512 instances, 2^10..2^20 evaluations (log-uniform), degree 2..4, sumcheck + "
                            "commit/open of each polynomial; python bench.py --workload batched for the full run"}
    # end to end: the same batch from pinned host memory (host->device copies inside)
    total = sum(i.polys.nbytes for i in insts)
    pinned = torch.empty(total, dtype=torch.uint8, pin_memory=True).numpy().view(np.uint64)
    host_insts, o = [], 0
    for i in insts:
        k = i.polys.size
        pinned[o:o + k] = i.polys.reshape(-1)
        host_insts.append(batch.Instance(pinned[o:o + k].reshape(i.polys.shape), i.index, QUERIES))
        o += k
    with ls_sched:
        batch.batch_prove(table, seed, host_insts, best, budget, engine=engine)
        e2e_times = [wall(lambda: batch.batch_prove(table, seed, host_insts, best, budget, engine=engine))
                     for _ in range(args.steps)]
    same_e2e = sum(np.array_equal(h.proof, a) for h, a in zip(host_insts, alone))

    step_s = statistics.mean(times)
    line = {"metric": "proofs/sec (mixed batch)", "value": count / step_s, "unit": "proofs/s", "n_gpus": 1,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": step_s * 1e3, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "u64 (Goldilocks)", "data": "synthetic",
            "config": {"workload": f"{count} instances: product sumcheck + Basefold commit/open_ext2 of every "
                                   "polynomial at the sumcheck point; 2^10..2^20 evaluations (log-uniform), "
                                   "degree in {2,3,4}, rate 1/2, 34 queries, table (22, 1, 22, seed 42)",
                       "instances": count, "evaluations": elems, "engine": engine, "workers": best, "coop_threshold": coop, "merkle_top_nodes": top,
                       "l2": "inputs larger than L2 (batch inputs resident in HBM)",
                       "timing": "host wall clock between device synchronisations (the batch spans one "
                                 "stream per worker)", "parallelism": "replicas x1"},
            "per_call": {"value": count / per_call_s, "unit": "proofs/s", "ms_per_step": per_call_s * 1e3,
                         "how": "every instance through gb_prove_instance, one after another, one stream"},
            "batched_over_per_call": per_call_s / step_s,
            "autotune_s": {f"{k[0]}w/{k[1]}/{k[2]}": round(v, 4) for k, v in tune.items()},
            "identical_to_per_call": {"service": f"{same}/{count}", "lockstep": f"{same_ls}/{count}",
                                      "host_inputs": f"{same_e2e}/{count}"},
            "engines": {"service": {"ms_per_step": statistics.mean(times_svc) * 1e3, "gpu_launches": int(launches_svc)},
                        "lockstep": {"ms_per_step": statistics.mean(times_ls) * 1e3, "gpu_launches": int(launches_ls),
                                     "commit_sumcheck_ms": phase[0].value, "open_ms": phase[1].value,
                                     "sumcheck_ms": phase[2].value, "schedule": lockstep_schedule},
                        "chosen": engine},
            "e2e": {"value": count / statistics.mean(e2e_times), "unit": "proofs/s",
                    "h2d_bytes_per_step": int(total),
                    "d2h_bytes_per_step": int(sum(i.proof.nbytes for i in insts))},
            "gpu_launches": int(launches), "clocks": clk.summary(),
            "step_ms_all": [round(t * 1e3, 2) for t in times]}
    print(json.dumps(line))


def run_served(args, summary=False):
    """Served matmul-layer jobs arriving as a Poisson stream.  The continuous prover service
    (prologues on worker streams, every opening in flight batched round by round in the open
    engines of its size class, HBM-budget admission) against the per-call path (one job at a time,
    in arrival order), both on the same arrival schedule; latency = arrival -> proof done.  Each
    offered load in `rates` gets its own schedule; the first is the headline load."""
    import torch
    from morpheus_gb300 import build as B
    B.build()
    from morpheus_gb300 import batch
    from morpheus_gb300.ajtai import AjtaiKey
    from morpheus_gb300.basefold import BasefoldTable
    seed = (0x452821E638D01377 % P, 0xBE5466CF34E90C6C % P)
    table = BasefoldTable.generate(24, LOG_RATE, 24, TABLE_SEED)
    key = AjtaiKey(np.array([0xA11CE, 1, 2, 3, 4, 5, 6, 7], np.uint32), 0, 16, 1024)
    warm, _ = batch.matmul_stream(3, seed=8, rate_per_s=args.rate, num_queries=QUERIES)
    for j in warm:
        batch.prove_matmul(table, key, seed, j)
    torch.cuda.synchronize()

    def pct(xs, q):
        return float(np.percentile(np.asarray(xs), q))

    def per_call(jobs, arrivals):
        # one job at a time, each starting once it has arrived and the previous one is done
        lat = []
        t0 = time.perf_counter()
        for j, a in zip(jobs, arrivals):
            now = time.perf_counter() - t0
            if now < a:
                time.sleep(a - now)
            batch.prove_matmul(table, key, seed, j)
            lat.append((time.perf_counter() - t0 - a) * 1e3)
        return time.perf_counter() - t0, lat

    slots = getattr(args, "slots", 0) or 0  # 0: no slot limit (the budget alone)

    def served(jobs, arrivals, continuous):
        with batch.ProverService(table, seed, QUERIES, workers=args.workers, hbm_budget=args.hbm_budget_gb << 30,
                                 continuous=continuous, slots=slots if continuous else None) as svc:
            svc.set_ajtai_key(key)
            for j in warm:
                svc.wait(svc.submit(j))
            tickets = []
            t0 = time.perf_counter()
            for j, a in zip(jobs, arrivals):
                now = time.perf_counter() - t0
                if now < a:
                    time.sleep(a - now)
                tickets.append(svc.submit(j))
            stats = [svc.wait(t)[1] for t in tickets]
            span = time.perf_counter() - t0
        return span, [st["latency_ms"] for st in stats]

    rates = [args.rate] + [r for r in getattr(args, "low_rates", []) if r != args.rate]
    runs = {}
    clk = None
    for rate in rates:
        jobs, arrivals = batch.matmul_stream(args.jobs, seed=7, rate_per_s=rate, num_queries=QUERIES)
        span_pc, lat_pc = per_call(jobs, arrivals)
        alone = [j.proof.copy() for j in jobs]
        for j in jobs:
            j.proof[:] = 0
        if rate == args.rate:
            with ClockSampler() as clk:
                span, lat = served(jobs, arrivals, True)
        else:
            span, lat = served(jobs, arrivals, True)
        same = sum(np.array_equal(j.proof, a) for j, a in zip(jobs, alone))
        run = {"offered_jobs_per_s": rate, "value": len(jobs) / span, "unit": "proofs/s",
               "p50_ms": pct(lat, 50), "p99_ms": pct(lat, 99), "max_ms": max(lat),
               "per_call": {"value": len(jobs) / span_pc, "p50_ms": pct(lat_pc, 50), "p99_ms": pct(lat_pc, 99)},
               "served_over_per_call": span_pc / span, "identical_to_per_call": f"{same}/{len(jobs)}"}
        if not summary:
            # the whole-job service (a worker proves a job start to end on its stream), same schedule
            for j in jobs:
                j.proof[:] = 0
            span_w, lat_w = served(jobs, arrivals, False)
            run["whole_job_service"] = {"value": len(jobs) / span_w, "p50_ms": pct(lat_w, 50),
                                        "p99_ms": pct(lat_w, 99),
                                        "identical": f"{sum(np.array_equal(j.proof, a) for j, a in zip(jobs, alone))}/"
                                                     f"{len(jobs)}"}
        runs[rate] = (run, jobs)
    head, jobs = runs[args.rate]
    others = [runs[r][0] for r in rates[1:]]
    workload = ("matmul-layer jobs (M, N, K in {256, 512, 1024, 4096}, int8), Poisson arrivals; continuous "
                "service (openings batched round by round in one engine per size class); python bench.py "
                "--workload served for the full run")
    if summary:
        out = {k: head[k] for k in ("value", "unit", "p50_ms", "p99_ms", "per_call", "served_over_per_call",
                                    "identical_to_per_call", "offered_jobs_per_s")}
        out.update({"jobs": len(jobs), "engine": "continuous", "workload": workload,
                    "below_capacity": [{k: o[k] for k in ("offered_jobs_per_s", "value", "p50_ms", "p99_ms",
                                                          "served_over_per_call", "identical_to_per_call")}
                                       for o in others]})
        return out
    h2d = sum(j.a.nbytes + j.b.nbytes for j in jobs)
    span = len(jobs) / head["value"]
    line = {"metric": "served proofs/sec", "value": head["value"], "unit": "proofs/s", "n_gpus": 1,
            "steps": len(jobs), "warmup": len(warm), "ms_per_step": span * 1e3 / len(jobs),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u64 (Goldilocks)",
            "data": "synthetic",
            "config": {"workload": f"{len(jobs)} matmul-layer jobs, Poisson arrivals at {args.rate:g}/s; "
                                   "M, N, K uniform over {256, 512, 1024, 4096}, int8 values; per job: Basefold "
                                   "commit of A and B, partial evaluation, degree-2 sumcheck over K, open of A "
                                   "and B (34 queries), Ajtai commit of a 2^16 witness (16 rows)",
                       "engine": "continuous (gb_prover_create_continuous)", "workers": args.workers,
                       "slots": slots,
                       "hbm_budget_gb": args.hbm_budget_gb, "offered_load_jobs_per_s": args.rate,
                       "table": "(24, 1, 24, seed 42)",
                       "timing": "host wall clock from the first arrival to the last proof",
                       "l2": "inputs larger than L2", "parallelism": "replicas x1"},
            "p50_ms": head["p50_ms"], "p99_ms": head["p99_ms"], "max_ms": head["max_ms"],
            "per_call": dict(head["per_call"], unit="proofs/s"),
            "served_over_per_call": head["served_over_per_call"],
            "identical_to_per_call": head["identical_to_per_call"],
            "whole_job_service": head.get("whole_job_service"),
            "other_loads": others,
            "e2e": {"value": head["value"], "unit": "proofs/s", "h2d_bytes_per_step": int(h2d / len(jobs)),
                    "d2h_bytes_per_step": int(sum(j.proof.nbytes for j in jobs) / len(jobs))},
            "clocks": clk.summary() if clk else None}
    print(json.dumps(line))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--num-vars", type=int, default=N_VARS)
    ap.add_argument("--no-extras", action="store_true", help="skip the roofline probes and the CPU baseline")
    ap.add_argument("--instances", type=int, default=512, help="batched workload: number of instances")
    ap.add_argument("--per-call-steps", type=int, default=1, help="batched workload: passes of the per-call path")
    ap.add_argument("--quick", action="store_true", help="batched workload: the lockstep engine only (profiling)")
    ap.add_argument("--jobs", type=int, default=200, help="served workload: number of jobs")
    ap.add_argument("--rate", type=float, default=200.0, help="served workload: mean arrivals per second")
    ap.add_argument("--slots", type=int, default=0, help="served workload: job slots of the continuous service "
                                                        "(0: no limit beside the HBM budget)")
    ap.add_argument("--low-rates", type=float, nargs="*", default=[80.0, 120.0],
                    help="served workload: further offered loads reported beside --rate")
    ap.add_argument("--workers", type=int, default=8, help="served workload: prover service workers")
    ap.add_argument("--hbm-budget-gb", type=int, default=96, help="served workload: admission budget")
    ap.add_argument("--witnesses", type=int, default=256, help="ajtai workload: witnesses per batch (1..256)")
    ap.add_argument("--ajtai-form", type=int, default=0, choices=[0, 1, 2, 3, 4],
                    help="ajtai workload: 0 by batch size, 1 witness-circulant GEMM, 2 key-Toeplitz GEMM, "
                         "3 key-Toeplitz GEMM on CTA pairs, 4 the pair GEMM on the key's Hankel windows")
    ap.add_argument("--workload", default="basefold", choices=["basefold", "sumcheck", "fold", "batch_open", "peval", "ajtai", "batched", "served"],
                    help="basefold (headline): commit+open proofs; sumcheck: 2 x 2^20 product sumcheck; "
                         "fold: one fused fold round over 2 x 2^24 Ext2; "
                         "batch_open: 8 polys x 2^20 opened at 2 points; "
                         "peval: fused permute + partial eval of 2^26 evaluations; "
                         "ajtai: 256 witnesses x 16 rows x 2^16 coefficients")
    args = ap.parse_args()
    if args.impl == "reference":
        return run_reference(args)
    if args.workload == "batched":
        return run_batched(args)
    if args.workload == "served":
        return run_served(args)
    if args.workload != "basefold":
        return run_side_workload(args)

    import torch
    from morpheus_gb300 import build as B
    B.build()
    from morpheus_gb300 import _native as Nn
    from morpheus_gb300.basefold import BasefoldCommitment, BasefoldTable
    from morpheus_gb300.memory import DeviceBuffer
    from morpheus_gb300.sumcheck import GpuLinearSumcheckProver, Transcript

    rank, world = env_rank()
    dist = world > 1
    if dist:
        import torch.distributed as tdist
        torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
        tdist.init_process_group("nccl")
    dev = torch.cuda.current_device()
    L = Nn.lib()
    stream = torch.cuda.Stream()
    L.gb_set_stream(ctypes.c_void_p(stream.cuda_stream))

    def ev_time(fn):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        fn()
        e1.record(stream)
        e1.synchronize()
        return e0.elapsed_time(e1)

    n = args.num_vars
    rng = np.random.default_rng(1234 + rank)
    ev_host = rng.integers(0, P, size=1 << n, dtype=np.uint64)
    pt = rng.integers(0, P, size=(n, 2), dtype=np.uint64)
    ev_dev = DeviceBuffer.from_numpy(ev_host)
    table = BasefoldTable.generate(n, LOG_RATE, n, TABLE_SEED)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)  # > L2 (129 MB)

    def step_device():
        c = BasefoldCommitment.commit(ev_dev, n, LOG_RATE)
        proof = c.open_ext2(pt, table, Transcript(b"bf-open"), QUERIES)
        return c, proof

    for _ in range(args.warmup):
        step_device()
    torch.cuda.synchronize()
    if dist:
        tdist.barrier()

    times, last = [], []
    with ClockSampler() as clk:
        l0 = L.gb_launch_count()
        for _ in range(args.steps):
            with torch.cuda.stream(stream):
                flush.zero_()
            times.append(ev_time(lambda: last.__setitem__(slice(None), [step_device()])))
        launches = (L.gb_launch_count() - l0) // max(1, args.steps)
        torch.cuda.synchronize()
        if dist:
            tdist.barrier()
        # e2e: pinned host evaluations through the C ABI, proof back to host memory
        ev_pinned = torch.from_numpy(ev_host.view(np.int64)).pin_memory()
        hptr = ev_pinned.data_ptr()
        proof_len = L.gb_basefold_proof_len(n, LOG_RATE, QUERIES)
        e2e_times = []
        for _ in range(args.steps):
            with torch.cuda.stream(stream):
                flush.zero_()
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            h = ctypes.c_void_p()
            root = np.zeros(4, np.uint64)
            Nn.check(L.gb_basefold_commit(None, ctypes.c_void_p(hptr), n, LOG_RATE, ctypes.byref(h),
                                          root.ctypes.data), "commit")
            c = BasefoldCommitment(h, n, LOG_RATE, root)
            c.open_ext2(pt, table, Transcript(b"bf-open"), QUERIES)
            e2e_times.append(time.perf_counter() - t0)
            del c
    ms_max, e2e_ms = max_over_ranks([statistics.mean(times), statistics.mean(e2e_times) * 1e3], dist, dev)
    value = replica_throughput(world, ms_max)

    extras = {}
    if not args.no_extras and rank == 0:
        # --- integer-pipe roofline of the dominant kernel (Poseidon2 Merkle layer over 2^21 parents)
        half = 1 << 21
        layer_in = DeviceBuffer(8 * half)
        layer_out = DeviceBuffer(4 * half)
        Nn.check(L.poseidon2_merkle_layer_ffi(layer_in.ptr, layer_out.ptr, half), "layer")
        lay_ms = min(ev_time(lambda: L.poseidon2_merkle_layer_ffi(layer_in.ptr, layer_out.ptr, half)) for _ in range(5))
        mulmods_per_perm = 520  # 8 external x 8 lanes x 4 + 22 internal x (4 + 8)
        achieved = half * mulmods_per_perm / (lay_ms * 1e-3) / 1e9
        blocks, iters = Nn.lib().gb_device_sm_count() * 8, 2048
        probe = DeviceBuffer(blocks * 256)
        Nn.check(L.gb_mulmod_probe(probe.ptr, blocks, iters), "probe")
        pr_ms = min(ev_time(lambda: L.gb_mulmod_probe(probe.ptr, blocks, iters)) for _ in range(5))
        peak = blocks * 256 * 8 * iters / (pr_ms * 1e-3) / 1e9
        extras["roofline"] = {
            "kernel": "merkle_level_kernel (Poseidon2 width 8, one permutation per thread)",
            "bound": "int", "achieved": achieved, "peak": peak, "unit": "Gmulmod/s", "frac": achieved / peak,
            "peak_source": "in-run probe: independent Goldilocks multiplication chains (gb_mulmod_probe); "
                           "neither hbm nor tensor bounds this kernel",
            "perms_per_s": half / (lay_ms * 1e-3), "launch_ms": lay_ms, "traffic": None,
        }
        # --- HBM roofline of the fused sumcheck fold round (2 polys x 2^24 Ext2 -> 2 x 2^23 Ext2)
        hbm_peak, src = measured_peaks()
        nf = 24
        src_buf = DeviceBuffer(2 * 2 * (1 << nf))
        dst_buf = DeviceBuffer(2 * 2 * (1 << (nf - 1)))
        msg = DeviceBuffer(16)
        work = DeviceBuffer(L.gb_sumcheck_round_workspace_words())
        work_np = np.zeros(work.len, np.uint64)
        Nn.check(L.cuda_memcpy_htod(work.ptr, work_np.ctypes.data, work.nbytes), "zero")
        pairs_out = 1 << (nf - 2)
        fr = lambda: L.gb_sumcheck_fold_round_ext2(src_buf.ptr, 0, 1 << nf, dst_buf.ptr, 1 << (nf - 1), 2,
                                                   pairs_out, 5, 7, msg.ptr, work.ptr)
        Nn.check(fr(), "fold round")
        fr_ms = min(ev_time(fr) for _ in range(5))
        fbytes = 2 * (1 << nf) * 16 + 2 * (1 << (nf - 1)) * 16
        extras["roofline_hbm"] = {
            "kernel": "sc_fold_round_e2_pf_kernel (fold 2 x 2^24 Ext2 + next round message)",
            "bound": "hbm", "achieved": fbytes / (fr_ms * 1e-3) / 1e9, "peak": hbm_peak, "unit": "GB/s",
            "frac": fbytes / (fr_ms * 1e-3) / 1e9 / hbm_peak, "peak_source": src, "bytes_per_launch": fbytes,
            "launch_ms": fr_ms,
        }
        # --- sumcheck Melem/s at the 2 x 2^20 shape (whole proof, host transcript)
        polys_host = rng.integers(0, P, size=(2, 1 << 20), dtype=np.uint64)
        polys = DeviceBuffer.from_numpy(polys_host.reshape(-1))
        sc_out = []

        def sc():
            t = Transcript(b"bench")
            sc_out.append(GpuLinearSumcheckProver(20, 2, t).prove((polys, 2), t))
        sc()
        sc_ms = statistics.median(ev_time(sc) for _ in range(5))
        extras["sumcheck_2x2^20"] = {"ms_per_proof": sc_ms, "melem_per_s": 2 * (1 << 20) / (sc_ms * 1e-3) / 1e6,
                                     "cpu_baseline": cpu_sumcheck_sample(polys_host, sc_out[-1].round_messages)}
        # --- Ajtai commitment at its configuration: 256 witnesses x 2^16 coefficients, rows 0..15
        flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")

        def ev_time_flushed(fn):
            with torch.cuda.stream(stream):
                flush.zero_()
            return ev_time(fn)
        extras["ajtai_c3"] = ajtai_c3_summary(L, Nn, DeviceBuffer, ev_time_flushed)
        del flush
        extras["cpu_baseline"] = cpu_baseline_sample(gpu_proof=last[-1][1], seed=1234 + rank)
        # the batched (512 mixed instances) and served (Poisson matmul jobs) configurations, compact
        L.gb_set_stream(None)
        extras["batched_512"] = run_batched(argparse.Namespace(instances=512, steps=1, warmup=1, per_call_steps=1),
                                            summary=True)
        extras["served"] = run_served(argparse.Namespace(jobs=100, rate=200.0, low_rates=[80.0], workers=8,
                                                         hbm_budget_gb=96), summary=True)

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": "proofs/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_max, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "u64 (Goldilocks)", "data": "synthetic",
            "config": {"workload": f"basefold commit+open_ext2, 2^{n} evals, rate 1/2, {QUERIES} queries",
                       "num_vars": n, "log_rate": LOG_RATE, "num_queries": QUERIES, "table_seed": TABLE_SEED,
                       "l2": "flushed between steps (256 MB write)", "parallelism": f"replicas x{world}"},
            "e2e": {"value": replica_throughput(world, e2e_ms), "unit": "proofs/s", "h2d_bytes_per_step": 8 << n,
                    "d2h_bytes_per_step": 8 * int(proof_len)},
            "gpu_launches": int(launches),
            "clocks": clk.summary(),
            "step_ms_all": [round(t, 3) for t in times],
        }
        line.update(extras)
        print(json.dumps(line))
    if dist:
        tdist.destroy_process_group()


if __name__ == "__main__":
    main()
