"""Dedicated tests of the reference's parity hazards that a restatement could
silently "fix": each test shows the quirk is live (it changes bits) and that
the port reproduces the reference's own code on it.  (The GPU side of each is
covered by the GPU tests against the same port and the golden fixtures.)"""
import ctypes
import json
import os

import numpy as np
import pytest

from conftest import GOLDEN
import circlecover_gb300 as cg
from circlecover_gb300 import workloads as W


def mul_scalar(lib, fn, lo, hi, s):
    f = getattr(lib, fn)
    f.argtypes = [ctypes.c_double, ctypes.c_double, ctypes.c_double, ctypes.c_void_p]
    out = np.zeros(2)
    f(lo, hi, s, out.ctypes.data)
    return out


def test_interval_times_scalar_rounds_upper_bound_down(port, ref):
    """interval.cuh:185-197: Interval * n with n >= 0 rounds BOTH bounds
    toward -inf (used for R = 0.61 * lambda and three other products)."""
    rng = np.random.default_rng(3)
    live = 0
    for _ in range(2000):
        lo = float(rng.uniform(0.5, 8.0))
        hi = lo + float(rng.uniform(0.0, 1.0))
        s = float(rng.choice([0.61, 0.25, 0.1 + rng.uniform(0, 1), -0.7]))
        a = mul_scalar(port.lib, "ccport_iv_mul_scalar", lo, hi, s)
        b = mul_scalar(ref.lib, "ccref_iv_mul_scalar", lo, hi, s)
        assert a.view(np.uint64).tolist() == b.view(np.uint64).tolist()
        if s >= 0:
            down = port.round(1, False, np.array([hi]), np.array([s]))[0]
            up = port.round(1, True, np.array([hi]), np.array([s]))[0]
            assert a[1] == down
            live += up != down
    assert live > 100  # the upper bound really is rounded the "wrong" way


def sb_task_box(lib, fn, parent, la_i, nla, r1_i, n1, r2_i, n2):
    f = getattr(lib, fn)
    f.argtypes = [ctypes.c_void_p] + [ctypes.c_int] * 6 + [ctypes.c_void_p]
    out = np.zeros(1, dtype=W.SB_BOX)
    p = np.ascontiguousarray(np.asarray(parent, dtype=W.SB_BOX).reshape(1))
    f(p.ctypes.data, la_i, nla, r1_i, n1, r2_i, n2, out.ctypes.data)
    return out


def test_r1_is_tightened_across_the_r2_loop(port, ref):
    """rectangle_size_bound.cu:281-291: r1 is declared once per r1 piece and
    r1.tighten_lb(r2.lb) accumulates over the r2 pieces visited before."""
    parent = W.sb_root(1.0, 2.5)
    nla, n1, n2 = 2, 8, 8
    changed = 0
    for la_i in range(nla):
        for r1_i in range(n1):
            first = sb_task_box(port.lib, "ccport_sb_task_box", parent, la_i, nla, r1_i, n1, 0, n2)
            for r2_i in range(n2):
                a = sb_task_box(port.lib, "ccport_sb_task_box", parent, la_i, nla, r1_i, n1, r2_i, n2)
                b = sb_task_box(ref.lib, "ccref_sb_task_box", parent, la_i, nla, r1_i, n1, r2_i, n2)
                assert np.array_equal(a.view(np.uint64), b.view(np.uint64))
                changed += a["r"][0, 0, 0] != first["r"][0, 0, 0]
    assert changed > 0  # the running tightening changes r1 for later r2 pieces


def test_criticals_come_out_in_the_canonical_order(golden_sb_prove_cases):
    """rectangle_size_bound.cu:103-130: the device appends criticals in any
    order; the result is the reference's sort (Variables::operator<) and
    merge, so lambda intervals ascend, and after the initial pass
    (merge over lambda only) no two criticals share a lambda interval."""
    for c in golden_sb_prove_cases:
        las = [(float.fromhex(b[0][0]), float.fromhex(b[0][1])) for b in c["criticals"]]
        assert las == sorted(las)
        if c["gens"] == 0:
            assert len(set(las)) == len(las)


@pytest.fixture(scope="module")
def golden_sb_prove_cases():
    with open(os.path.join(GOLDEN, "sb_prove_golden.json")) as f:
        return json.load(f)["cases"]


def test_trap_sites_mark_boxes_instead_of_aborting(port):
    """A reference trap() kills the whole run; here the box is flagged and
    never certified.  The golden size-bound masks reach trap sites, and the
    boxes that do are certified by no criterion that trapped."""
    z = np.load(os.path.join(GOLDEN, "sb_eval_golden.npz"))
    masks = z["masks"]
    trapped = masks[(masks >> 31) & 1 == 1]
    assert len(trapped) > 0
    got = port.sb_eval(np.ascontiguousarray(z["boxes"]).view(W.SB_BOX).reshape(-1), threads=8)
    assert np.array_equal(got, masks)
