"""Generate tests/golden/reference_vectors.json from the reference tree.

Run here (where the reference sources exist), never on the GPU machine:

    python tests/golden/make_golden.py --ref <reference checkout>

Two kinds of vectors are written:

* golden values stated in the reference's own tests, read from the test files
  as text (each entry records file:line and the literal it was read from);
* outputs of the reference's own code, built for the host from its sources by
  oracle/Makefile into oracle/_ref/ (Poseidon2 / Goldilocks / Ext2 device code
  and the Ajtai ChaCha8 PRG + CPU reference).

The GPU tests and the CPU oracle tests both check against this file, so it
travels with the repository while the reference tree does not.
"""
import argparse
import ctypes
import json
import os
import re
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
P = 0xFFFFFFFF00000001
Q = 0xFFFFFFFEFFFFFFE1
C_AGL = 0x10000001F
HALF_AGL = 0x7FFFFFFF7FFFFFF1


def find_line(path, literal):
    with open(path) as f:
        for i, line in enumerate(f, 1):
            if literal in line:
                return i
    raise SystemExit(f"literal {literal!r} not found in {path}")


def text_vectors(ref):
    out = {}
    # Poseidon2 width-8 KAT printed by the reference's standalone test.
    f = os.path.join(ref, "cuda/poseidon2_kernels.cu")
    src = open(f).read()
    m = re.search(r"uint64_t expected\[8\] = \{([^}]*)\}", src)
    vals = [int(x.strip().rstrip("ULL")) for x in m.group(1).replace("\n", " ").split(",") if x.strip()]
    out["poseidon2_plonky3_kat"] = {
        "source": f"cuda/poseidon2_kernels.cu:{find_line(f, 'uint64_t expected[8]')}",
        "input": list(range(8)),
        "expected": vals,
        "note": "The reference's permutation (same constants in cuda/poseidon2.cuh, "
                "goldilocks-cuda-rs/src/cpu_poseidon2.rs, zk-torch-3/src/transcript.rs) does not "
                "produce this vector; the reference's own code output is in poseidon2_ref.",
    }
    # almost-Goldilocks golden add/mul cases (hand-computed in the test).
    f = os.path.join(ref, "cuda_almost_goldilocks/almost_field_test.cu")
    sym = {"AGL_PRIME": Q, "ALMOST_REDUCE_C": C_AGL, "ALMOST_HALF_P_PLUS_ONE": HALF_AGL}

    def ev(expr):
        e = expr.strip().replace("ULL", "")
        for k, v in sym.items():
            e = e.replace(k, str(v))
        e = e.replace("0xFFFFFFFFFFFFFFFF", str(2**64 - 1))
        return int(eval(e, {"__builtins__": {}}))  # arithmetic on literals only

    src = open(f).read()
    adds = re.search(r"AddCase add_cases\[\] = \{(.*?)\};", src, re.S).group(1)
    muls = re.search(r"MulCase mul_cases\[\] = \{(.*?)\};", src, re.S).group(1)

    def cases(block):
        res = []
        for line in block.splitlines():
            line = line.split("//")[0]
            mm = re.search(r"\{([^{}]*)\}", line)
            if mm:
                res.append([ev(x) for x in mm.group(1).split(",")])
        return res

    out["agl_add_golden"] = {"source": f"cuda_almost_goldilocks/almost_field_test.cu:{find_line(f, 'AddCase add_cases')}",
                             "cases": cases(adds)}
    out["agl_mul_golden"] = {"source": f"cuda_almost_goldilocks/almost_field_test.cu:{find_line(f, 'MulCase mul_cases')}",
                             "cases": cases(muls)}
    f = os.path.join(ref, "cuda_almost_goldilocks/almost_extension_test.cu")
    ln = find_line(f, "(1 + 2X)(3 + 4X)")
    assert "27 + 10X" in open(f).read()
    out["aext2_mul_golden"] = {"source": f"cuda_almost_goldilocks/almost_extension_test.cu:{ln}",
                               "cases": [[[1, 2], [3, 4], [27, 10]], [[2, 3], [2, 3], [31, 12]]]}
    f = os.path.join(ref, "zk-torch-3/src/sumcheck/linear_prover.rs")
    ln = find_line(f, "1*5 + 2*6 + 3*7 + 4*8 = 5 + 12 + 21 + 32 = 70")
    out["sumcheck_h70"] = {"source": f"zk-torch-3/src/sumcheck/linear_prover.rs:{ln}",
                           "p1": [1, 2, 3, 4], "p2": [5, 6, 7, 8], "sum": 70,
                           "labels": {"base": "test", "ext2": "test_cpu_ext2"}}
    # Monolith-12 permutation KAT and the Merkle test codewords of the reference's CPU tests
    f = os.path.join(ref, "goldilocks-cuda-rs/src/cpu_monolith.rs")
    src = open(f).read()
    m = re.search(r"let expected: \[u64; 12\] = \[(.*?)\];", src, re.S)
    kat = [int(x) for x in re.findall(r"\d+", m.group(1))]
    assert len(kat) == 12
    m = re.search(r"let codeword: Vec<u64> = vec!\[(.*?)\];", src, re.S)
    big = [int(x, 16) for x in re.findall(r"0x[0-9A-Fa-f]+", m.group(1))]
    assert len(big) == 32
    m = re.search(r"let cw: Vec<u64> = vec!\[(.*?)\];", src, re.S)
    specific = [int(x) for x in re.findall(r"\d+", m.group(1))]
    out["monolith_kat"] = {"source": f"goldilocks-cuda-rs/src/cpu_monolith.rs:{find_line(f, 'let expected: [u64; 12]')}",
                           "input": list(range(12)), "expected": kat}
    out["monolith_tree_inputs"] = {
        "source": f"goldilocks-cuda-rs/src/cpu_monolith.rs:{find_line(f, 'fn test_monolith_gpu_vs_cpu_merkle()')}",
        "codewords": [list(range(100, 108)), list(range(1, 33)), specific, big],
        "ext2_codeword": [10, 20, 30, 40, 50, 60, 70, 80],
        "large_value_state": [8, P - 8] + [0] * 10}
    f = os.path.join(ref, "zk-torch-3/src/commit/basefold.rs")
    ln = find_line(f, "num_queries: 34")
    out["basefold_key_default"] = {"source": f"zk-torch-3/src/commit/basefold.rs:{ln}",
                                   "log_rate": 3, "num_queries": 34, "seed": 42}
    return out


def ref_vectors():
    u64p = np.ctypeslib.ndpointer(dtype=np.uint64, flags="C_CONTIGUOUS")
    u32p = np.ctypeslib.ndpointer(dtype=np.uint32, flags="C_CONTIGUOUS")
    G = ctypes.CDLL(os.path.join(REPO, "oracle/_ref/libgl_ref.so"))
    A = ctypes.CDLL(os.path.join(REPO, "oracle/_ref/libajtai_ref.so"))
    G.ref_poseidon2_init()
    G.ref_poseidon2_permute.argtypes = [u64p]
    for nm in ("ref_gl_mul", "ref_gl_add", "ref_gl_sub"):
        getattr(G, nm).restype = ctypes.c_uint64
        getattr(G, nm).argtypes = [ctypes.c_uint64, ctypes.c_uint64]
    G.ref_ext2_mul.argtypes = [u64p, u64p, u64p]
    A.ref_chacha8_block.argtypes = [u32p, ctypes.c_uint32, u32p, u32p]
    A.ref_ring_elem.argtypes = [u32p, ctypes.c_int, ctypes.c_uint64, u64p]
    A.ref_commit_wide.argtypes = [u32p, u64p, ctypes.c_uint64, ctypes.c_uint64, ctypes.c_int, ctypes.c_int, u64p]
    A.ref_commit_binary.argtypes = [u32p, u64p, ctypes.c_uint64, u64p]

    rng = np.random.default_rng(20261203)
    out = {}
    ins = [np.arange(8, dtype=np.uint64), np.zeros(8, np.uint64),
           np.full(8, P - 1, np.uint64), np.full(8, 2**64 - 1, np.uint64)]
    ins += [rng.integers(0, 2**64, size=8, dtype=np.uint64, endpoint=False) for _ in range(12)]
    p2 = []
    for s in ins:
        o = s.copy()
        G.ref_poseidon2_permute(o)
        p2.append([[int(x) for x in s], [int(x) for x in o]])
    out["poseidon2_ref"] = {"source": "cuda/poseidon2.cuh:322-362 built for the host (oracle/_ref/libgl_ref.so)",
                            "cases": p2}
    edge = [0, 1, 2, P - 1, P, P + 1, 2**64 - 1, 2**32, 2**32 - 1, 2**63]
    pairs = [(a, b) for a in edge for b in edge]
    pairs += [tuple(int(x) for x in rng.integers(0, 2**64, size=2, dtype=np.uint64)) for _ in range(64)]
    out["gl_ops_ref"] = {"source": "cuda/goldilocks.cuh:182-311 built for the host; outputs canonicalised",
                         "cases": [[a, b, int(G.ref_gl_add(a, b)), int(G.ref_gl_sub(a, b)), int(G.ref_gl_mul(a, b))]
                                   for a, b in pairs]}
    e2 = []
    for _ in range(32):
        a = rng.integers(0, P, size=2, dtype=np.uint64)
        b = rng.integers(0, P, size=2, dtype=np.uint64)
        o = np.zeros(2, np.uint64)
        G.ref_ext2_mul(a, b, o)
        e2.append([[int(x) for x in a], [int(x) for x in b], [int(x) for x in o]])
    out["ext2_mul_ref"] = {"source": "cuda/extension.cuh:113-125 built for the host", "cases": e2}

    cc = []
    for key, ctr, nonce in [([1, 2, 3, 4, 5, 6, 7, 8], 0, [42, 1000, 1]), ([1, 2, 3, 4, 5, 6, 7, 8], 1, [42, 1000, 1]),
                            ([0] * 8, 0, [0, 0, 0]), ([0xFFFFFFFF] * 8, 7, [3, 5, 7])]:
        o = np.zeros(16, np.uint32)
        A.ref_chacha8_block(np.array(key, np.uint32), ctr, np.array(nonce, np.uint32), o)
        cc.append([key, ctr, nonce, [int(x) for x in o]])
    out["chacha8_ref"] = {"source": "cuda_almost_goldilocks/ajtai_chacha8.cuh:60-98", "cases": cc}
    key = np.array([9, 8, 7, 6, 5, 4, 3, 2], np.uint32)
    ring = []
    for row, j in [(0, 0), (3, 77), (41, 1023), (15, 2**33 + 5)]:
        o = np.zeros(64, np.uint64)
        A.ref_ring_elem(key, row, j, o)
        ring.append([row, j, [int(x) for x in o]])
    out["ajtai_ring_elem_ref"] = {"source": "cuda_almost_goldilocks/ajtai_cpu_reference.cuh:124-148",
                                  "key": [int(x) for x in key], "cases": ring}
    N = 4
    z = rng.integers(0, Q, size=N * 64, dtype=np.uint64)
    o = np.zeros(42 * 64, np.uint64)
    A.ref_commit_wide(key, z, N, 3, 0, 42, o)
    out["ajtai_commit_wide_ref"] = {"source": "cpu_prg_ring_elem<64> + cpu_ring_mul<64> (ajtai_cpu_reference.cuh:78-148)",
                                    "key": [int(x) for x in key], "N": N, "col_offset": 3, "rows": 42,
                                    "z": [int(x) for x in z], "out": [int(x) for x in o]}
    z8 = rng.integers(0, 256, size=N * 64, dtype=np.uint64)
    o = np.zeros(16 * 64, np.uint64)
    A.ref_commit_wide(key, z8, N, 0, 0, 16, o)
    out["ajtai_commit_u8_ref"] = {"source": "as ajtai_commit_wide_ref, witness entries in [0, 256), rows 0..15",
                                  "key": [int(x) for x in key], "N": N, "rows": 16,
                                  "z": [int(x) for x in z8], "out": [int(x) for x in o]}
    bits = rng.integers(0, 2**64, size=3, dtype=np.uint64)
    o = np.zeros(42 * 64, np.uint64)
    A.ref_commit_binary(key, bits, 3, o)
    out["ajtai_commit_binary_ref"] = {"source": "cpu_ajtai_commit<64, 42> (ajtai_cpu_reference.cuh:157-181)",
                                      "key": [int(x) for x in key], "z_bits": [int(x) for x in bits],
                                      "out": [int(x) for x in o]}
    return out


def _sha(a):
    import hashlib
    return hashlib.sha256(np.ascontiguousarray(a, dtype="<u8").tobytes()).hexdigest()


def basefold_kernel_vectors():
    """Basefold commitments made by the reference's own kernels (cuda/basefold.cuh and the Merkle
    kernels of goldilocks-cuda-rs/cuda/wrapper.cu) run on the host by oracle/_ref/libbasefold_ref.so,
    on the seeded inputs of tests/seeded_inputs.py (so the GPU machine can regenerate the inputs)."""
    sys.path.insert(0, os.path.dirname(HERE))
    import seeded_inputs as SI
    u64p = np.ctypeslib.ndpointer(dtype=np.uint64, flags="C_CONTIGUOUS")
    R = ctypes.CDLL(os.path.join(REPO, "oracle/_ref/libbasefold_ref.so"))
    R.ref_bf_init()
    R.ref_basefold_commit.argtypes = [u64p, ctypes.c_int, ctypes.c_int, u64p, u64p, u64p, u64p]
    cases = []
    for n, lr in [(1, 1), (4, 1), (6, 3), (13, 1), (16, 2), (22, 1)]:
        ev, _ = SI.c2_inputs(n)
        L = 1 << (n + lr)
        cw, bh = np.zeros(L, np.uint64), np.zeros(1 << n, np.uint64)
        tree, root = np.zeros((L - 1) * 4, np.uint64), np.zeros(4, np.uint64)
        R.ref_basefold_commit(ev, n, lr, cw, bh, tree, root)
        P_ = np.uint64(P)
        cw, bh, tree, root = cw % P_, bh % P_, tree % P_, root % P_  # canonical, as the reference compares
        case = {"num_vars": n, "log_rate": lr, "evals_sha256": _sha(ev), "root": [int(x) for x in root],
                "codeword_sha256": _sha(cw), "bh_evals_sha256": _sha(bh), "tree_sha256": _sha(tree)}
        if L <= 64:
            case["codeword"] = [int(x) for x in cw]
        cases.append(case)
    return {"source": "cuda/basefold.cuh:57-205 (bit reverse, interpolation, encode) and "
                      "goldilocks-cuda-rs/cuda/wrapper.cu:934-960, 1604-1710 (leaf hashes, tree layers), "
                      "launched as wrapper.cu:1242-1313 and :1653-1710 do and in the order of "
                      "BasefoldCommitment::commit_device (goldilocks-cuda-rs/src/basefold.rs:380-410); "
                      "run on the host by oracle/_ref/libbasefold_ref.so",
            "inputs": "tests/seeded_inputs.py c2_inputs(num_vars)",
            "cases": cases}


def basefold_open_vectors():
    """Openings made by the reference's kernels (open_ext2's launch sequence, basefold.rs:578-870,
    restated around them; the transcript is the oracle's restatement of zk-torch-3's Transcript)."""
    sys.path.insert(0, os.path.dirname(HERE))
    sys.path.insert(0, REPO)
    import oracle as O
    import seeded_inputs as SI
    O.set_threads(os.cpu_count() or 1)
    cases = []

    def record(name, evals, n, lr, point, table_vars, q, label, u64_after_label, explicit):
        comm = O.ref_basefold_commit(evals, lr)
        table = O.basefold_table(table_vars, lr, table_vars, 42)
        t = O.Transcript(label)
        if u64_after_label is not None:
            t.append_u64(b"", u64_after_label)
        proof = O.ref_basefold_open_ext2(comm, point, table, t, q)
        head = 2 + 6 * n + 4 * (n - 1) + (2 << lr)
        case = {"name": name, "num_vars": n, "log_rate": lr, "table_vars": table_vars, "table_seed": 42,
                "num_queries": q, "label": label.decode(), "u64_after_label": u64_after_label,
                "evals_sha256": _sha(evals), "point": [int(x) for x in np.asarray(point).reshape(-1)],
                "root": [int(x) for x in comm["root"]], "proof_len": int(proof.size),
                "proof_sha256": _sha(proof), "proof_head": [int(x) for x in proof[:head]]}
        if explicit:
            case["evals"] = [int(x) for x in evals]
            case["proof"] = [int(x) for x in proof]
        cases.append(case)

    # the reference's own GPU-against-CPU opening test, its inputs exactly
    # (zk-torch-3/src/commit/cpu_basefold.rs:433-509)
    ev = np.array([(P - 1 - i * 1000 % P) % P for i in range(64)], np.uint64)
    pt = np.array([[100 + i, 0] for i in range(6)], np.uint64)
    record("cpu_vs_gpu_opening", ev, 6, 3, pt, 9, 10, b"test-open", 42, True)
    # the C2 shape (seeded inputs of tests/seeded_inputs.py), rate 1/2, 34 queries
    for n in (4, 13, 16, 22):
        ev, pt = SI.c2_inputs(n)
        record(f"c2_shape_n{n}", ev, n, 1, pt, n, 34, b"bf-open", None, n <= 4)
    return {"source": "open_ext2 (goldilocks-cuda-rs/src/basefold.rs:578-870) with the reference's kernels "
                      "(cuda/basefold.cuh, cuda/eq_lagrange.cuh, wrapper.cu Merkle kernels) run on the host by "
                      "oracle/_ref/libbasefold_ref.so; launch sizes of wrapper.cu:1223-1600; commitment from "
                      "the reference's kernels too",
            "cases": cases}


def sumcheck_vectors():
    """Ext2-challenge product sumchecks made by the reference's kernels (cuda/sumcheck_prover.cuh,
    launched as wrapper.cu:1751-1785 in GpuSumcheckStateExt2's sequence) on seeded inputs."""
    sys.path.insert(0, os.path.dirname(HERE))
    sys.path.insert(0, REPO)
    import oracle as O
    import seeded_inputs as SI
    cases = []
    shapes = [("c1", SI.C1["seed"], 2, 20, SI.C1["label"]), ("d3_n12", 0x5C3, 3, 12, b"bench"),
              ("d4_n10", 0x5C4, 4, 10, b"bench"), ("d8_n6", 0x5C8, 8, 6, b"bench")]
    for name, seed, d, n, label in shapes:
        polys = SI.field_elems(seed, d << n).reshape(d, 1 << n)
        r = O.ref_sumcheck_prove_ext2(O.Transcript(label), polys)
        cases.append({"name": name, "seed": seed, "degree": d, "num_vars": n, "label": label.decode(),
                      "polys_sha256": _sha(polys),
                      "round_messages": [int(x) for x in r["round_messages"].reshape(-1)],
                      "challenges": [int(x) for x in r["challenges"].reshape(-1)],
                      "final_evals": [int(x) for x in r["final_evals"].reshape(-1)],
                      "final_eval": [int(x) for x in r["final_eval"]]})
    return {"source": "GpuLinearSumcheckProver::prove (zk-torch-3/src/sumcheck/gpu_prover.rs:36-90) on "
                      "GpuSumcheckStateExt2 (goldilocks-cuda-rs/src/sumcheck_prover.rs:215-410) with the "
                      "reference's kernels run on the host by oracle/_ref/libbasefold_ref.so; inputs "
                      "tests/seeded_inputs.py field_elems(seed, d << n)",
            "cases": cases}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", default=os.environ.get("MORPHEUS_REFERENCE"),
                    help="the reference checkout (default: $MORPHEUS_REFERENCE)")
    args = ap.parse_args()
    if not args.ref or not os.path.isdir(args.ref):
        sys.exit("reference tree not found; fixtures are generated only where it exists")
    subprocess.run(["make", "-s", "-C", os.path.join(REPO, "oracle"), "all", "ref", f"REF={args.ref}"], check=True)
    data = {"generated_by": "tests/golden/make_golden.py"}
    data.update(text_vectors(args.ref))
    data.update(ref_vectors())
    with open(os.path.join(HERE, "reference_vectors.json"), "w") as f:
        json.dump(data, f, indent=0)
    print("wrote", os.path.join(HERE, "reference_vectors.json"))
    with open(os.path.join(HERE, "reference_basefold.json"), "w") as f:
        json.dump({"generated_by": "tests/golden/make_golden.py",
                   "basefold_commit_ref": basefold_kernel_vectors(),
                   "basefold_open_ref": basefold_open_vectors(),
                   "sumcheck_ref": sumcheck_vectors()}, f, indent=0)
    print("wrote", os.path.join(HERE, "reference_basefold.json"))


if __name__ == "__main__":
    main()
