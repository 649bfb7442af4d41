"""Node reads per query of the reference traversals on the benchmark
workloads, measured with the instrumented CPU restatement (test
infrastructure: feeds the algorithmic byte counts of bench.py's roofline).

    python oracle/visit_counts.py   ->  profiles/visit_counts.json
"""

import json
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

from oracle import oracle as o  # noqa: E402


def main(n=10_000_000, nq_sample=20_000, k=16):
    points = np.random.default_rng(3).random((n, 3), dtype=np.float32)
    queries = np.random.default_rng(12).random((n, 3), dtype=np.float32)
    tree = o.OracleTree(points)
    sample = queries[np.linspace(0, n - 1, nq_sample).astype(np.int64)]
    vi, vl = o.visit_counts(tree, 0, sample, k=k)
    r = np.float32((32 * 3 / (4 * np.pi * n)) ** (1 / 3))
    spheres = np.concatenate([sample, np.full((nq_sample, 1), r, np.float32)], axis=1)
    si, sl = o.visit_counts(tree, 1, spheres, kind=o.KIND_SPHERE)
    out = {
        "workload": "uniform [0,1)^3, points seed 3, queries seed 12 (bench.py inputs)",
        "n": n,
        "k": k,
        "sample_queries": nq_sample,
        "internal": vi,
        "leaves": vl,
        "radius": float(r),
        "spatial_internal": si,
        "spatial_leaves": sl,
        "how": "instrumented verbatim ArborX traversals of oracle/abx_oracle.c (abxo_visit_counts)",
    }
    path = os.path.join(ROOT, "profiles", "visit_counts.json")
    with open(path, "w") as f:
        json.dump(out, f, indent=1)
    print(json.dumps(out))


if __name__ == "__main__":
    main()
