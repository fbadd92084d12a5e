"""GPU tier: the size-bound proof at the sizes of its full runs against the
reference's own criteria (tests/golden/sb_full_proof_golden.json, made by
tests/golden/make_sb_proof_golden.py with oracle/_ref/libccref.so): single
tasks of the initial pass of the reference's own size-bound proof (lambda in
[1, 2.5], 256 x 128 x 128 tasks, r3..r6 in 64) and of the run over lambda in
[1, 8] (1024 x 256 x 128 tasks), through cc_sb_generation, with and without
the FP32 pre-filter.  Criticals (all bits), flags, trace digest, per-level
outcome counts and leaf counts are bit-exact."""
import json
import os

import numpy as np
import pytest

from circlecover_gb300 import workloads as W

pytestmark = pytest.mark.gpu

FIXTURE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "sb_full_proof_golden.json")


def sb_from_hex(rows):
    out = np.zeros(len(rows), dtype=W.SB_BOX)
    for i, r in enumerate(rows):
        out[i]["la"] = (float.fromhex(r[0][0]), float.fromhex(r[0][1]))
        for k in range(6):
            out[i]["r"][k] = (float.fromhex(r[k + 1][0]), float.fromhex(r[k + 1][1]))
    return out


@pytest.mark.parametrize("run", ["reference", "lambda_1_8"])
def test_sampled_tasks_equal_the_reference(prover, run):
    fx = json.load(open(FIXTURE))["runs"][run]
    root = sb_from_hex([fx["root"]])
    leaves = 0
    for t in fx["tasks"]:
        for fp32 in (True, False):
            crit, flags, st = prover.sb_generation(root, 0, fx["la_splits"], fx["r_splits"], t["lo"], t["hi"], fp32=fp32)
            where = (run, t["lo"], fp32)
            want = sb_from_hex(t["criticals"])
            assert len(crit) == len(want) and np.array_equal(crit.view(np.uint64), want.view(np.uint64)), where
            assert [int(f) for f in flags] == t["flags"], where
            assert st["digest"] == t["digest"], where
            assert st["task_counts"] == t["task_counts"] and st["cell_counts"] == t["cell_counts"], where
            assert st["leaf_counts"] == t["leaf_counts"] and st["leaf_evals"] == t["leaf_evals"], where
            assert st["cert_failures"] == 0, where
        leaves += t["leaf_evals"]
    assert leaves > 0
