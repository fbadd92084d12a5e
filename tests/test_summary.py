"""Max_distances (kernel_compute_distance_from_theoretical_worst_cases,
tight_rectangle.cu:322-456): the prover's per-box items + in-order fold
against a restatement of the reference's kernel on the reference's own
interval code (CPU), and the GPU's parallel items + fold against both."""
import ctypes

import numpy as np
import pytest

import circlecover_gb300 as cg
from circlecover_gb300 import workloads as W
from conftest import boxes_from_hex


def near_worst_cases(n, seed):
    """Critical-like boxes around the 2- and 3-disk worst cases."""
    rng = np.random.default_rng(seed)
    b = np.zeros(n, dtype=W.TIGHT_BOX)
    lam = rng.uniform(1.0, 2.08, n)
    w = 10.0 ** rng.uniform(-7, -3, n)
    two = rng.random(n) < 0.5
    w3 = (16 * lam ** 4 + 40 * lam ** 2 + 9) / (256 * lam ** 2)
    r1 = np.where(two, 0.25 * (lam ** 2 + 1), w3) * (1 + rng.uniform(-1e-3, 1e-3, n))
    r2 = np.where(two, 0.25, w3) * (1 + rng.uniform(-1e-3, 1e-3, n))
    r3 = np.where(two, rng.uniform(0, 0.05, n), w3 * (1 + rng.uniform(-1e-3, 1e-3, n)))
    b["la"][:, 0], b["la"][:, 1] = lam, lam + w
    for k, r in enumerate((r1, r2, r3)):
        b["r"][:, k, 0], b["r"][:, k, 1] = r, r + w
    b["r"][:, 3, 0], b["r"][:, 3, 1] = 0.0, w
    return b


def summary_bytes(lib, fn, boxes):
    out = cg.CcTightSummary()
    f = getattr(lib, fn)
    f.argtypes = [ctypes.c_void_p, ctypes.c_size_t, ctypes.POINTER(cg.CcTightSummary)]
    boxes = np.ascontiguousarray(boxes, dtype=W.TIGHT_BOX)
    f(boxes.ctypes.data if len(boxes) else None, len(boxes), ctypes.byref(out))
    return bytes(out)


def test_port_summary_matches_reference(ref, port, golden_prove):
    cases = [near_worst_cases(2000, 1), near_worst_cases(7, 2), np.zeros(0, dtype=W.TIGHT_BOX)]
    cases += [boxes_from_hex(c["criticals"]) for c in golden_prove if c["criticals"]]
    for boxes in cases:
        assert summary_bytes(port.lib, "ccport_tight_summary", boxes) == summary_bytes(ref.lib, "ccref_tight_summary", boxes)


def test_summary_fields_are_filled(port):
    s = cg.CcTightSummary.from_buffer_copy(summary_bytes(port.lib, "ccport_tight_summary", near_worst_cases(500, 3)))
    assert s.have_range_2d and s.have_range_3d
    assert s.pocket_width_3d > -1.0 and s.dist_r1_3d.lb < 0 < s.dist_r1_3d.ub


@pytest.mark.gpu
def test_gpu_summary_matches_port(prover, port, golden_prove):
    cases = [near_worst_cases(100_000, 4), near_worst_cases(3, 5)]
    cases += [boxes_from_hex(c["criticals"]) for c in golden_prove if c["criticals"]]
    for boxes in cases:
        assert bytes(prover.tight_summary(boxes)) == summary_bytes(port.lib, "ccport_tight_summary", boxes)
