"""Generate tests/golden/config_goldens.json: the oracle's outputs at the full C2 configuration.

    python tests/golden/make_config_goldens.py

C2 is one Basefold commit + open_ext2 of 2^22 evaluations (rate 1/2, 34 queries, folding table
(22, 1, 22, seed 42)) on the seeded inputs of tests/seeded_inputs.py.  The oracle (oracle/oracle.c)
takes about two minutes for it on one thread, so the GPU tests compare against these fixtures
instead of rerunning it: SHA-256 digests of the codeword, the tree, the table and the whole proof,
plus the root, the tree's top levels, the proof's head (evaluation, round oracles, folded roots,
final codeword) and the query indices written out in full, so that a mismatch shows where.
"""
import hashlib
import json
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, REPO)
sys.path.insert(0, os.path.dirname(HERE))

import oracle as O  # noqa: E402
import seeded_inputs as SI  # noqa: E402


def sha(a):
    return hashlib.sha256(np.ascontiguousarray(a, dtype="<u8").tobytes()).hexdigest()


def ints(a):
    return [int(x) for x in np.asarray(a).reshape(-1)]


def proof_head_len(n, lr):
    return 2 + 6 * n + 4 * (n - 1) + (2 << lr)


def query_indices(proof, n, lr, q):
    per_q = 1 + 4 * n + 4 * sum(n + lr - 1 - r for r in range(n))
    base = proof_head_len(n, lr)
    return [int(proof[base + k * per_q]) for k in range(q)]


def c2_fixture(n):
    cfg = SI.C2
    lr, q = cfg["log_rate"], cfg["num_queries"]
    ev, pt = SI.c2_inputs(n)
    t0 = time.time()
    ent, off = O.basefold_table(n, lr, n, cfg["table_seed"])
    c = O.basefold_commit(ev, lr)
    proof = O.basefold_open_ext2(c, pt, (ent, off), O.Transcript(cfg["label"]), q)
    assert O.basefold_verify_ext2(c["root"], n, lr, pt, proof, q, (ent, off), O.Transcript(cfg["label"]))
    tree = c["tree"].reshape(-1, 4)
    top = min(31, tree.shape[0])
    print(f"n={n}: {time.time() - t0:.1f} s", file=sys.stderr)
    return {
        "num_vars": n, "log_rate": lr, "num_queries": q, "table_seed": cfg["table_seed"],
        "label": cfg["label"].decode(), "input_seed": cfg["seed"] + n,
        "evals_sha256": sha(ev), "point": ints(pt),
        "root": ints(c["root"]),
        "codeword_sha256": sha(c["codeword"]), "tree_sha256": sha(c["tree"]),
        "tree_top_nodes": ints(tree[-top:]),
        "table_entries_sha256": sha(ent), "table_level_offsets": ints(off),
        "proof_len": int(proof.size), "proof_sha256": sha(proof),
        "proof_head": ints(proof[:proof_head_len(n, lr)]),
        "query_indices": query_indices(proof, n, lr, q),
    }


def main():
    O.build(ref_root="")
    O.set_threads(os.cpu_count() or 1)
    data = {"generated_by": "tests/golden/make_config_goldens.py",
            "oracle": "oracle/oracle.c (CPU restatement; bit-exact)",
            "c2": c2_fixture(SI.C2["num_vars"]),
            "c2_n16": c2_fixture(16)}
    path = os.path.join(HERE, "config_goldens.json")
    with open(path, "w") as f:
        json.dump(data, f, indent=0)
    print("wrote", path)


if __name__ == "__main__":
    main()
