"""Generate the golden fixtures of the tight-rectangle path from the
REFERENCE's own criteria code (oracle/_ref/libccref.so, built from the
reference sources by oracle/ref/Makefile).  Run where the reference sources
exist:

    python tests/golden/make_golden.py

Outputs (committed, small):
  tight_eval_golden.npz   boxes + verdict masks + per-box op counts
  tight_prove_golden.json small proofs: root, split counts, critical boxes
                          (hex floats), trace counts and digest
  sb_eval_golden.npz      size-bound boxes + verdict masks + op counts
  sb_prove_golden.json    small size-bound proofs (as tight_prove_golden)
The boxes come from circlecover_gb300.workloads (seeded, platform-independent)
plus hand-made edge cases.
"""
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from circlecover_gb300 import workloads as W  # noqa: E402
from oracle import oracle as O  # noqa: E402

DBL_MAX = np.finfo(np.float64).max


def edge_boxes():
    """Degenerate and boundary inputs the reference's own runs can produce:
    point intervals, lambda at 1 and at lambda_2 and at the proof's upper end,
    radii ranges [0, DBL_MAX], zero-width and empty radius intervals, the
    2- and 3-disk worst cases."""
    rows = []
    l2 = W.LAMBDA_2
    lam_hi = W.TIGHT_LAMBDA_MAX

    def box(la, r):
        b = np.zeros(1, dtype=W.TIGHT_BOX)
        b["la"][0] = la
        b["r"][0] = r
        rows.append(b[0])

    for la in [(1.0, 1.0), (1.0, 1.0 + 2 ** -20), (l2, l2), (l2 - 1e-3, l2 + 1e-3), (lam_hi, lam_hi), (2.0, lam_hi)]:
        lam = 0.5 * (la[0] + la[1])
        w3 = (16 * lam ** 4 + 40 * lam ** 2 + 9) / (256 * lam ** 2)  # 3-disk worst case
        w2a, w2b = 0.25 * (lam * lam + 1.0), 0.25  # 2-disk worst case
        box(la, [(0.0, DBL_MAX)] * 4)
        box(la, [(w3, w3), (w3, w3), (w3, w3), (0.0, 0.0)])
        box(la, [(w3 - 1e-4, w3 + 1e-4), (w3 - 1e-4, w3 + 1e-4), (w3 - 1e-4, w3 + 1e-4), (0.0, 1e-4)])
        box(la, [(w2a, w2a), (w2b, w2b), (0.0, 0.05), (0.0, 0.05)])
        box(la, [(w2a - 1e-3, w2a), (w2b - 1e-3, w2b), (0.0, 1e-3), (0.0, 1e-3)])
        box(la, [(0.9, 0.9), (0.1, 0.1), (0.0, 0.0), (0.0, 0.0)])
        box(la, [(0.3, 0.2), (0.1, 0.2), (0.0, 0.1), (0.0, 0.1)])  # empty r1 interval
        box(la, [(0.0, 0.0)] * 4)
        box(la, [(1e-300, 1e-300), (1e-310, 1e-310), (5e-324, 5e-324), (0.0, 0.0)])  # tiny and subnormal
        box(la, [(0.26, 0.27), (0.26, 0.27), (0.25, 0.27), (0.2, 0.25)])
    return np.array(rows, dtype=W.TIGHT_BOX)


def sb_edge_boxes():
    """Size-bound boxes at the edges: all radii at the bound 9/64, point
    intervals, zero radii, lambda at 1, 2.5 and 8, R close to 0."""
    rows = []
    ub = 9.0 / 64.0

    def box(la, r):
        b = np.zeros(1, dtype=W.SB_BOX)
        b["la"][0] = la
        b["r"][0] = r
        rows.append(b[0])

    for la in [(1.0, 1.0), (1.0, 1.0 + 2 ** -20), (2.5, 2.5), (1.5, 1.6), (8.0, 8.0), (2.4, 2.5)]:
        lam = la[1]
        box(la, [(0.0, ub)] * 6)
        box(la, [(ub, ub)] * 6)
        box(la, [(ub - 1e-3, ub)] * 6)
        box(la, [(0.0, 0.0)] * 6)
        box(la, [(ub, ub), (ub, ub), (0.1, 0.1), (0.05, 0.05), (0.01, 0.02), (0.0, 0.01)])
        w = 0.61 * lam / 6.0
        w = min(w, ub)
        box(la, [(w - 1e-6, w)] * 6)
        box(la, [(0.13, 0.14), (0.12, 0.13), (0.11, 0.12), (0.1, 0.11), (0.09, 0.1), (0.08, 0.09)])
        box(la, [(0.2, 0.1)] + [(0.0, 0.01)] * 5)  # empty r1
        for r3 in (0.0, 0.002):  # r1, r2 in opposite corners, a tiny rest
            box(la, [(0.119, 0.12), (0.119, 0.12)] + [(r3, r3)] + [(0.0, r3)] * 3)
    return np.array(rows, dtype=W.SB_BOX)


PROOF_CASES = [
    # (name, la range, la_init, r_init, gens, r_gen)
    ("near_one", (1.0, 1.0 + 0.1 / 256), 2, (16, 16, 16, 16), (1, 2), (16, 16, 16, 8)),
    ("mid", (1.5, 1.51), 2, (32, 32, 16, 16), (2,), (16, 16, 16, 16)),
    ("two_disk", (2.0, W.TIGHT_LAMBDA_MAX), 4, (16, 16, 16, 16), (1, 1), (16, 16, 8, 8)),
    ("config1_slice", (1.0, 1.1), 4, (8, 16, 16, 16), (1, 2, 2), (16, 16, 16, 8)),
]


UB_W = 9.0 / 64.0
# (name, lambda range, radius ranges (None = [0, 9/64] each), grid: la_init, r_init, la_gen, r_gen, gens)
SB_PROOF_CASES = [
    ("init_small", (1.0, 2.5), None, (4, (8, 8, 4, 4, 4, 4), 64, (32, 32, 16, 16, 16, 32), 0)),
    ("three_generations", (1.0, 2.5), None, (4, (8, 8, 4, 4, 4, 4), 2, (2, 2, 2, 2, 2, 2), 3)),
    ("wide_lambda", (2.5, 8.0), None, (4, (8, 8, 4, 4, 4, 4), 2, (2, 2, 2, 2, 2, 4), 1)),
    ("mid_lambda", (1.2, 1.6), None, (4, (16, 16, 8, 6, 6, 6), 2, (2, 2, 2, 2, 2, 2), 1)),
    ("large_disks", (1.0, 1.1), [(0.12, UB_W), (0.1, UB_W)] + [(0.0, UB_W)] * 4,
     (2, (8, 8, 6, 6, 6, 6), 64, (32, 32, 16, 16, 16, 32), 0)),
    ("mixed_disks", (1.2, 1.5), [(0.12, UB_W), (0.11, UB_W), (0.1, 0.13), (0.0, 0.12), (0.0, 0.1), (0.0, 0.1)],
     (2, (4, 4, 4, 4, 4, 4), 2, (2, 2, 2, 2, 2, 2), 1)),
]


def sb_root_box(la, radii):
    b = np.zeros(1, dtype=W.SB_BOX)
    b["la"][0] = la
    b["r"][0] = radii if radii is not None else [(0.0, UB_W)] * 6
    return b[0]


def hexbox6(b):
    return [[float(b["la"][0]).hex(), float(b["la"][1]).hex()]] + [[float(b["r"][k][0]).hex(), float(b["r"][k][1]).hex()]
                                                                   for k in range(6)]


def hexbox(b):
    return [[float(b["la"][0]).hex(), float(b["la"][1]).hex()]] + [[float(b["r"][k][0]).hex(), float(b["r"][k][1]).hex()]
                                                                   for k in range(4)]


def main():
    O.ensure_built()
    ref = O.Ref()
    parts = [W.tight_microbench(4096, seed=1), W.tight_near_critical(4096, seed=5), edge_boxes()]
    boxes = np.concatenate(parts)
    masks, ops = ref.tight_eval(boxes, threads=8, count_ops=True)
    np.savez_compressed(os.path.join(HERE, "tight_eval_golden.npz"), boxes=boxes.view(np.float64).reshape(len(boxes), 10),
                        masks=masks, ops=ops, parts=np.array([len(p) for p in parts]))
    print("eval fixtures:", len(boxes), "boxes")

    # algorithmic work of the bench workload: the reference's directed-rounding
    # operation count per box on the first 2**16 boxes of the 2**24-box
    # microbench (seed 1), the sample the bench scales its roofline from
    bench = W.tight_microbench(1 << 16, seed=1)
    bm, bops = ref.tight_eval(bench, threads=8, count_ops=True)
    assert bops.max() < 65536
    # the share of each box's work done by the two bisection passes (the
    # strip-width and gap-width kernels): the port's count of those loops,
    # which execute the reference's operations one for one; the main pass
    # gets the rest of the reference's count
    p3 = O.Port(count=True).tight_eval_passes(bench)
    assert np.all(p3[:, 1] + p3[:, 2] <= bops)
    np.savez_compressed(os.path.join(HERE, "tight_bench_ops.npz"), ops=bops.astype(np.uint16), masks=bm,
                        cover_ops=p3[:, 1].astype(np.uint16), gaps_ops=p3[:, 2].astype(np.uint16))
    print("bench sample: mean ops/box %.1f (strip bisection %.1f, gap bisection %.1f)"
          % (bops.mean(), p3[:, 1].mean(), p3[:, 2].mean()))

    # size-bound criteria: per-box masks of the reference's code
    sb_parts = [W.sb_boxes(2000, seed=3, la_hi=2.5), W.sb_boxes(1500, seed=4, la_hi=8.0), sb_edge_boxes()]
    sbb = np.concatenate(sb_parts)
    sbm, sbops = ref.sb_eval(sbb, threads=8, count_ops=True)
    np.savez_compressed(os.path.join(HERE, "sb_eval_golden.npz"), boxes=sbb.view(np.float64).reshape(len(sbb), 14),
                        masks=sbm, ops=sbops, parts=np.array([len(p) for p in sb_parts]))
    print("size-bound eval fixtures:", len(sbb), "boxes, mean ops %.0f" % sbops.mean())

    cases = []
    for name, la, la_init, r_init, gens, r_gen in PROOF_CASES:
        root = W.tight_root(*la)
        g = O.make_grid(la_init, r_init, gens, r_gen)
        crit, st = ref.tight_prove(root, g, threads=8)
        cases.append(dict(name=name, root=hexbox(root), la_init=la_init, r_init=list(r_init), gens=list(gens),
                          r_gen=list(r_gen), criticals=[hexbox(b) for b in crit], stats=st))
        print("proof", name, "criticals", len(crit), "gen sizes", st["gen_sizes"], "leaves", st["leaf_evals"])
    with open(os.path.join(HERE, "tight_prove_golden.json"), "w") as f:
        json.dump(dict(source="reference criteria built for the host (oracle/_ref)", cases=cases), f, indent=0)

    from circlecover_gb300 import make_sb_grid
    sb_cases = []
    for name, la, radii, (la_init, r_init, la_gen, r_gen, gens) in SB_PROOF_CASES:
        root = sb_root_box(la, radii)
        g = make_sb_grid(la_init, r_init, la_gen, r_gen, gens)
        crit, flags, st = ref.sb_prove(root, g, threads=8)
        sb_cases.append(dict(name=name, root=hexbox6(root), la_init=la_init, r_init=list(r_init), la_gen=la_gen,
                             r_gen=list(r_gen), gens=gens, criticals=[hexbox6(b) for b in crit],
                             flags=[int(x) for x in flags], stats=st))
        print("size-bound proof", name, "criticals", len(crit), "trapped", int(flags.sum()), "gen sizes",
              st["gen_sizes"], "leaves", st["leaf_evals"])
    with open(os.path.join(HERE, "sb_prove_golden.json"), "w") as f:
        json.dump(dict(source="reference criteria built for the host (oracle/_ref)", cases=sb_cases), f, indent=0)


if __name__ == "__main__":
    main()
