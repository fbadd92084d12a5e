"""Size-bound proof (rectangle_size_bound::find_critical_intervals): the host
restatement of the driver on the port against the reference's own run
(golden fixtures, and the live reference library where it exists), and the
GPU engine (cc_sb_prove) against both.  Criticals are compared bit for bit in
the reference's final order (sorted and merged), together with the trap
flags, the per-level outcome counts and the trace digest."""
import json
import os

import numpy as np
import pytest

from conftest import GOLDEN
import circlecover_gb300 as cg
from circlecover_gb300 import workloads as W

UB_W = 9.0 / 64.0


@pytest.fixture(scope="module")
def golden_sb_prove():
    with open(os.path.join(GOLDEN, "sb_prove_golden.json")) as f:
        return json.load(f)["cases"]


def box6_from_hex(h):
    b = np.zeros(1, dtype=W.SB_BOX)
    b["la"][0] = (float.fromhex(h[0][0]), float.fromhex(h[0][1]))
    for k in range(6):
        b["r"][0, k] = (float.fromhex(h[k + 1][0]), float.fromhex(h[k + 1][1]))
    return b[0]


def boxes6_from_hex(rows):
    if not rows:
        return np.zeros(0, dtype=W.SB_BOX)
    return np.array([box6_from_hex(r) for r in rows], dtype=W.SB_BOX)


def grid_of(c):
    return cg.make_sb_grid(c["la_init"], c["r_init"], c["la_gen"], c["r_gen"], c["gens"])


def check_against(c, crit, flags, st):
    want = boxes6_from_hex(c["criticals"])
    assert len(crit) == len(want)
    assert np.array_equal(crit.view(np.uint64), want.view(np.uint64))
    assert [int(x) for x in flags] == c["flags"]
    for k in ("task_counts", "cell_counts", "leaf_counts", "digest", "leaf_evals", "trapped_leaves",
              "trapped_shortcuts", "gen_sizes", "generations_run"):
        assert st[k] == c["stats"][k], k


CASES = range(6)


def test_golden_cases_cover_the_driver(golden_sb_prove):
    """The fixtures exercise several generations (all three merge widths),
    both shortcut levels, trapped leaves and most criteria of the cascade."""
    assert max(c["gens"] for c in golden_sb_prove) >= 3
    leaf = np.sum([c["stats"]["leaf_counts"] for c in golden_sb_prove], axis=0)
    task = np.sum([c["stats"]["task_counts"] for c in golden_sb_prove], axis=0)
    cell = np.sum([c["stats"]["cell_counts"] for c in golden_sb_prove], axis=0)
    assert task[1] > 0 and task[3] > 0
    assert cell[1] > 0 and cell[3] > 0
    assert leaf[cg.SBT_LEAF_TRAPPED] > 0 and leaf[cg.SBT_LEAF_CRITICAL] > 0
    assert (leaf[:14] > 0).sum() >= 11


@pytest.mark.parametrize("case", CASES)
def test_port_matches_golden_sb_proofs(port, golden_sb_prove, case):
    c = golden_sb_prove[case]
    crit, flags, st = port.sb_prove(box6_from_hex(c["root"]), grid_of(c), threads=8)
    check_against(c, crit, flags, st)


def test_port_matches_reference_live_sb_proof(ref, port):
    root = np.zeros(1, dtype=W.SB_BOX)[0]
    root["la"] = (1.05, 1.3)
    root["r"] = [(0.1, UB_W), (0.05, UB_W), (0.0, 0.12), (0.0, 0.1), (0.0, 0.1), (0.0, 0.1)]
    g = cg.make_sb_grid(3, (6, 6, 4, 4, 4, 4), 2, (2, 2, 2, 2, 2, 2), 2)
    a = ref.sb_prove(root, g, threads=8)
    b = port.sb_prove(root, g, threads=8)
    assert np.array_equal(a[0].view(np.uint64), b[0].view(np.uint64))
    assert np.array_equal(a[1], b[1])
    assert a[2] == b[2]


def test_driver_is_independent_of_thread_count(port, golden_sb_prove):
    c = golden_sb_prove[3]
    one = port.sb_prove(box6_from_hex(c["root"]), grid_of(c), threads=1)
    many = port.sb_prove(box6_from_hex(c["root"]), grid_of(c), threads=13)
    assert np.array_equal(one[0].view(np.uint64), many[0].view(np.uint64))
    assert one[2] == many[2]


@pytest.mark.gpu
@pytest.mark.parametrize("case", CASES)
def test_gpu_sb_prove_matches_golden(prover, golden_sb_prove, case):
    c = golden_sb_prove[case]
    crit, flags, st = prover.sb_find_critical_intervals(box6_from_hex(c["root"]), grid_of(c))
    check_against(c, crit, flags, st)
    if st["leaf_evals"]:
        assert st["kernel_launches"] > 0


@pytest.mark.gpu
@pytest.mark.parametrize("form", ["plain", "no_fp32"])
def test_gpu_sb_prove_other_forms_match_golden(prover, golden_sb_prove, form):
    """The plain form (whole cascade per thread) and the batched form without
    the FP32 pre-filter give the same criticals, flags and trace."""
    for c in golden_sb_prove:
        crit, flags, st = prover.sb_find_critical_intervals(box6_from_hex(c["root"]), grid_of(c),
                                                            plain=form == "plain", fp32=False)
        check_against(c, crit, flags, st)
        assert st["fp32_decided"] == 0


@pytest.mark.gpu
def test_gpu_fp32_prefilter_decides_only_empty_leaves(prover, golden_sb_prove):
    decided = 0
    for c in golden_sb_prove:
        crit, flags, st = prover.sb_find_critical_intervals(box6_from_hex(c["root"]), grid_of(c))
        assert st["fp32_decided"] <= st["leaf_counts"][cg.SBT_LEAF_EMPTY]
        decided += st["fp32_decided"]
        if st["widening_samples"]:
            assert 1.0 <= st["widening_mean"] <= st["widening_max"]
    assert decided > 0


@pytest.mark.gpu
def test_gpu_sb_prove_matches_port_larger(prover, port):
    """Several leaf slices and task chunks: the reference's own initial grid
    restricted to a narrow lambda range, one generation."""
    root = W.sb_root(1.0, 1.02)
    g = cg.make_sb_grid(2, (32, 32, 16, 12, 12, 12), 2, (4, 4, 4, 4, 4, 4), 1)
    a = port.sb_prove(root, g, threads=16)
    b = prover.sb_find_critical_intervals(root, g)
    assert np.array_equal(a[0].view(np.uint64), b[0].view(np.uint64))
    assert np.array_equal(a[1], b[1])
    for k, v in a[2].items():
        assert b[2][k] == v, k


@pytest.mark.gpu
def test_gpu_sb_prove_small_work_units(prover, golden_sb_prove, monkeypatch):
    """Tiny task chunks and leaf slices: many chunks, slices and critical
    drains give the same criticals and trace."""
    monkeypatch.setenv("CC_SB_TASK_CHUNK_LOG2", "3")
    monkeypatch.setenv("CC_SB_SLICE_LOG2", "9")
    for case in (1, 3, 4):
        c = golden_sb_prove[case]
        crit, flags, st = prover.sb_find_critical_intervals(box6_from_hex(c["root"]), grid_of(c))
        check_against(c, crit, flags, st)


@pytest.mark.gpu
def test_gpu_sb_prove_rejects_bad_grid(prover):
    root = W.sb_root(1.0, 2.5)
    for bad in [cg.make_sb_grid(0, (4,) * 6), cg.make_sb_grid(4, (4, 4, 4, 4, 4, 2048)),
                cg.make_sb_grid(4, (4,) * 6, 0, (4,) * 6, 1)]:
        with pytest.raises(cg.CudaError):
            prover.sb_find_critical_intervals(root, bad)
