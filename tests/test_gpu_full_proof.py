"""GPU tier: the tight proof at full size against the reference's own
criteria (tests/golden/tight_full_proof_golden.json, made by
tests/golden/make_proof_golden.py with oracle/_ref/libccref.so).

Two roots: the full tight_rectangle proof (lambda in [1,
2.0898841580413818342], 256 lambda pieces, r splits 128^4, the reference's
refinement schedule; tight_rectangle.cu:44-70, 458-498) and the small
plain-method workload (lambda in [1, 1.1], r1 in 64 pieces).

* Every generation is compared on the fixture's sampled task ranges, run
  from the fixture's parents: in generation 0 every task that produced
  criticals on the GPU (at most eight) and two seeded others, in each
  refinement generation one task; critical boxes (all 160 bits), trace
  digest, per-outcome counts and leaf count.
* Every generation run whole from its parents reproduces the next
  generation's parents stored in the fixture, and the whole proof in one
  call (batched and learned forms) ends as the generations do.
"""
import json
import os

import numpy as np
import pytest

import circlecover_gb300 as cg
from circlecover_gb300 import workloads as W

pytestmark = pytest.mark.gpu

FIXTURE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "tight_full_proof_golden.json")


def boxes_from_hex(rows):
    out = np.zeros(len(rows), dtype=W.TIGHT_BOX)
    for i, r in enumerate(rows):
        out[i]["la"] = (float.fromhex(r[0][0]), float.fromhex(r[0][1]))
        for k in range(4):
            out[i]["r"][k] = (float.fromhex(r[k + 1][0]), float.fromhex(r[k + 1][1]))
    return out


@pytest.fixture(scope="module")
def fixture():
    with open(FIXTURE) as f:
        return json.load(f)


def same_boxes(a, b):
    return len(a) == len(b) and np.array_equal(np.ascontiguousarray(a).view(np.uint64),
                                               np.ascontiguousarray(b).view(np.uint64))


@pytest.mark.parametrize("name", ["full", "config1"])
def test_oracle_ranges_of_every_generation(prover, fixture, name):
    checked = 0
    for e in fixture[name]["generations"]:
        parents = boxes_from_hex(e["parents"])
        for o in e["oracle"]:
            crit, st = prover.tight_generation(parents, e["la_splits"], e["r_splits"], o["lo"], o["hi"])
            want = boxes_from_hex(o["criticals"])
            where = (name, e["gen"], o["lo"], o["hi"])
            assert same_boxes(crit, want), where
            assert st["digest"] == o["digest"], where
            assert st["counts"] == o["counts"], where
            assert st["leaf_evals"] == o["leaf_evals"], where
            assert st["trapped_leaves"] == o["trapped"], where
            checked += 1
    # the initial pass has its oracle result whole
    assert checked >= 1 and fixture[name]["generations"][0]["oracle"]


@pytest.mark.parametrize("name", ["full", "config1"])
def test_whole_generations_and_proof(prover, fixture, name):
    gens = fixture[name]["generations"]
    sizes = []
    for e in gens:
        parents = boxes_from_hex(e["parents"])
        crit, st = prover.tight_generation(parents, e["la_splits"], e["r_splits"])
        assert same_boxes(crit, boxes_from_hex(e["gpu_criticals"])), (name, e["gen"])
        sizes.append(len(crit))
        assert st["cert_failures"] == 0
    # the whole proof in one call, batched and learned
    fx = fixture[name]
    root = boxes_from_hex([fx["root"]])[0]
    sched = fixture["schedule"]
    grid = cg.make_grid(fx["la_splits_init"], fx["r_splits_init"], sched["la_splits_gen"], sched["r_splits_gen"])
    crit, st = prover.tight_find_critical_intervals(root, grid)
    assert st["gen_sizes"] == sizes and len(crit) == sizes[-1]
    assert st["cert_failures"] == 0 and st["fp32_first"][3] == 0
    prover.mlp_init(5)
    crit_l, st_l = prover.tight_find_critical_intervals(root, grid, learned=True)
    assert same_boxes(crit_l, crit) and st_l["gen_sizes"] == sizes and st_l["leaf_evals"] == st["leaf_evals"]
