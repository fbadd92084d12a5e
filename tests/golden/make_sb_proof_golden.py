"""ORACLE / TEST INFRASTRUCTURE ONLY: golden fixtures of the size-bound proof
at the sizes of the full runs.

Writes tests/golden/sb_full_proof_golden.json: for the reference's own
size-bound proof (lambda in [1, 2.5], 256 x 128 x 128 tasks, r3..r6 in 64;
rectangle_size_bound/rectangle_size_bound.cu:36-62, 312-382) and for the run
over lambda in [1, 8] (1024 lambda pieces x 256 r1 pieces, r2 and r3..r6 as
the reference), a seeded sample of single tasks of the initial pass -- a
task is (lambda piece, r1 piece, r2 piece) in the order of the reference's
host loops (:276-310) -- with the oracle's merged criticals (hex floats),
flags, trace digest, per-outcome counts and leaf count, computed by the
restated driver (oracle/sb_driver.hpp) on the REFERENCE's own criteria
(oracle/_ref/libccref.so, built from the reference sources).  The sample
draws tasks from lambda pieces across the range, favouring the hard end
(lambda near 1), and keeps tasks of every outcome.

  python tests/golden/make_sb_proof_golden.py [THREADS]
"""
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from circlecover_gb300 import workloads as W  # noqa: E402

OUT = os.path.join(HERE, "sb_full_proof_golden.json")
RUNS = {
    "reference": ((1.0, 2.5), 256, (128, 128, 64, 64, 64, 64)),
    "lambda_1_8": ((1.0, 8.0), 1024, (256, 128, 64, 64, 64, 64)),
}
SEED = 20261205
# lambda pieces to sample from, per run (fractions of the lambda split count)
PIECES = (0.0, 0.0, 0.004, 0.03, 0.1, 0.25, 0.5, 0.9)


def box_hex(b):
    return [[float(b["la"][0]).hex(), float(b["la"][1]).hex()]] + \
        [[float(b["r"][k][0]).hex(), float(b["r"][k][1]).hex()] for k in range(6)]


def main(threads):
    from oracle import oracle as O
    O.ensure_built()
    ref = O.Ref()
    rng = np.random.default_rng(SEED)
    fx = {"note": "single tasks of the initial pass (generation 0) of each run; task = (lambda piece * r1 "
                  "splits + r1 piece) * r2 splits + r2 piece", "runs": {}}
    for name, ((la_lo, la_hi), nla, rs) in RUNS.items():
        root = W.sb_root(la_lo, la_hi)
        per_la = rs[0] * rs[1]
        entries = []
        for frac in PIECES:
            la_i = min(nla - 1, int(frac * nla))
            task = la_i * per_la + int(rng.integers(0, per_la))
            crit, flags, st = ref.sb_generation(np.array([root]), 0, nla, rs, task, task + 1, threads=threads)
            entries.append({"lo": task, "hi": task + 1, "criticals": [box_hex(b) for b in crit],
                            "flags": [int(f) for f in flags], "digest": st["digest"],
                            "task_counts": st["task_counts"], "cell_counts": st["cell_counts"],
                            "leaf_counts": st["leaf_counts"], "leaf_evals": st["leaf_evals"]})
            print(name, task, la_i, st["task_counts"], st["leaf_evals"], len(crit), flush=True)
        fx["runs"][name] = {"root": box_hex(root), "la_splits": nla, "r_splits": list(rs), "tasks": entries}
    with open(OUT, "w") as f:
        json.dump(fx, f, indent=1)
    print("wrote", OUT)


if __name__ == "__main__":
    main(int(sys.argv[1]) if len(sys.argv) > 1 else (os.cpu_count() or 4))
