"""ORACLE / TEST INFRASTRUCTURE ONLY: golden fixtures of the tight proof at
the sizes of the workloads that the bench and the GPU tests run.

Writes tests/golden/tight_full_proof_golden.json for two roots:

* "full": the full tight_rectangle proof, the reference's root lambda in
  [1, 2.0898841580413818342] and schedule (tight_rectangle/tight_rectangle.cu:
  44-70, 458-498): 256 lambda pieces, r splits 128^4, then refinement
  generations with lambda splits 1,2,2,2,... and r splits 128^3 x 64;
* "config1": the small plain-method workload, lambda in [1, 1.1] with r1 in
  64 pieces, same refinement schedule.

Per generation the fixture holds its parents and, for task ranges of that
generation, the oracle's criticals (hex floats), trace digest, per-outcome
counts and leaf count, computed by the restated driver (oracle/
tight_driver.hpp) on the REFERENCE's own criteria (oracle/_ref/libccref.so,
built from the reference sources).  The CPU evaluates about 4e4 leaves per
second on 8 cores, so no generation is run whole: generation 0 (2.7e6 to
3.9e6 leaves per task) is sampled by every task that produced criticals on
the GPU (at most GEN0_HOT) and GEN0_RANDOM seeded others; a refinement
generation (1.3e8 leaves per task, about an hour each) by one task that
produced criticals on the GPU, else a seeded one.  The parents of
generation 1 and later are the GPU's output of the previous generation,
stored as they are ("parents_source"); the ranges that produced them are
among the sampled ones.

Steps (the second one takes hours on 8 cores; it resumes from the partial
file it writes after every range, generation 0 of both roots first):

  python tests/golden/make_proof_golden.py import DIR   # GPU lists <root>_genNN.npy
  python tests/golden/make_proof_golden.py run [THREADS]
"""
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from circlecover_gb300 import workloads as W  # noqa: E402

OUT = os.path.join(HERE, "tight_full_proof_golden.json")
GENS = (1, 2, 2, 2, 2, 1, 2, 1, 2, 1, 2)
R_GEN = (128, 128, 128, 64)
ROOTS = {"full": ((1.0, W.TIGHT_LAMBDA_MAX), 256, (128, 128, 128, 128)),
         "config1": ((1.0, 1.1), 256, (64, 128, 128, 128))}
SAMPLE_SEED = 20261204
SAMPLES_PER_GEN = 1
GEN0_HOT = 8
GEN0_RANDOM = 2


def box_hex(b):
    return [[float(b["la"][0]).hex(), float(b["la"][1]).hex()]] + \
        [[float(b["r"][k][0]).hex(), float(b["r"][k][1]).hex()] for k in range(4)]


def boxes_from_hex(rows):
    out = np.zeros(len(rows), dtype=W.TIGHT_BOX)
    for i, r in enumerate(rows):
        out[i]["la"] = (float.fromhex(r[0][0]), float.fromhex(r[0][1]))
        for k in range(4):
            out[i]["r"][k] = (float.fromhex(r[k + 1][0]), float.fromhex(r[k + 1][1]))
    return out


def task_of(parents, la_splits, crit):
    """Task (parent * la_splits + lambda piece) whose lambda piece and r1
    range contain each critical box (the first such task)."""
    from oracle import oracle as O
    port = O.Port()
    tasks = []
    for c in crit:
        found = -1
        for p, par in enumerate(parents):
            if not (par["r"][0][0] <= c["r"][0][0] and c["r"][0][1] <= par["r"][0][1]):
                continue
            for j in range(la_splits):
                lo, hi = port.subinterval(float(par["la"][0]), float(par["la"][1]), j, la_splits)
                if lo == c["la"][0] and hi == c["la"][1]:
                    found = p * la_splits + j
                    break
            if found >= 0:
                break
        tasks.append(found)
    return tasks


def import_gpu(src):
    fx = {"note": "parents: generation 0's root is the reference's; later parents are the GPU's output of the "
                  "previous generation (parents_source), checked against the oracle on the ranges below",
          "schedule": {"la_splits_gen": list(GENS), "r_splits_gen": list(R_GEN)}}
    rng = np.random.default_rng(SAMPLE_SEED)
    for name, ((la_lo, la_hi), la0, r0) in ROOTS.items():
        root = W.tight_root(la_lo, la_hi)
        gens = []
        parents = np.array([root])
        g = 0
        while len(parents):
            la = la0 if g == 0 else GENS[g - 1]
            rs = r0 if g == 0 else R_GEN
            path = os.path.join(src, "%s_gen%02d.npy" % (name, g))
            out = np.load(path) if os.path.exists(path) else None
            n_tasks = len(parents) * la
            entry = {"gen": g, "la_splits": la, "r_splits": list(rs), "n_tasks": n_tasks,
                     "parents": [box_hex(b) for b in parents],
                     "parents_source": "reference root" if g == 0 else "GPU output of generation %d" % (g - 1)}
            if out is not None:
                entry["gpu_criticals"] = [box_hex(b) for b in out]
            hot = sorted({t for t in task_of(parents, la, out) if t >= 0}) if out is not None else []
            want = GEN0_HOT + GEN0_RANDOM if g == 0 else SAMPLES_PER_GEN
            pick = list(hot[:GEN0_HOT if g == 0 else SAMPLES_PER_GEN])
            others = [t for t in range(n_tasks) if t not in pick]
            while len(pick) < want and others:
                t = int(rng.choice(others))
                others.remove(t)
                pick.append(t)
            entry["ranges"] = [[t, t + 1] for t in sorted(pick)]
            entry["oracle"] = []
            gens.append(entry)
            if out is None or not len(out):
                break
            parents = out
            g += 1
        fx[name] = {"root": box_hex(root), "la_splits_init": la0, "r_splits_init": list(r0), "generations": gens}
    with open(OUT, "w") as f:
        json.dump(fx, f, indent=1)
    print("wrote", OUT)


def run(threads):
    from oracle import oracle as O
    O.ensure_built()
    ref = O.Ref()
    fx = json.load(open(OUT))
    # generation 0 of every root first, then the refinement generations
    order = sorted(((e["gen"], name, e) for name in ROOTS for e in fx[name]["generations"]), key=lambda x: x[:2])
    for _, name, entry in order:
        done = {(o["lo"], o["hi"]) for o in entry["oracle"]}
        parents = boxes_from_hex(entry["parents"])
        for lo, hi in entry["ranges"]:
            if (lo, hi) in done:
                continue
            crit, st = ref.tight_generation(parents, entry["la_splits"], entry["r_splits"], lo, hi,
                                            threads=threads)
            entry["oracle"].append({"lo": lo, "hi": hi, "criticals": [box_hex(b) for b in crit],
                                    "digest": st["digest"], "counts": st["counts"],
                                    "leaf_evals": st["leaf_evals"], "trapped": st["trapped_leaves"]})
            with open(OUT, "w") as f:
                json.dump(fx, f, indent=1)
            print(name, entry["gen"], lo, hi, len(crit), st["leaf_evals"], flush=True)


if __name__ == "__main__":
    if len(sys.argv) >= 3 and sys.argv[1] == "import":
        import_gpu(sys.argv[2])
    elif len(sys.argv) >= 2 and sys.argv[1] == "run":
        run(int(sys.argv[2]) if len(sys.argv) > 2 else (os.cpu_count() or 4))
    else:
        print(__doc__)
        sys.exit(2)
