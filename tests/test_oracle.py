"""CPU tier: the oracle itself.

* the host directed-rounding layer (error-free transforms) equals fesetround
  on random and special operands;
* the CPU port of the prover's criteria reproduces the golden fixtures that
  the reference's own code produced (always), and the live reference library
  on fresh random boxes and proofs (where the reference sources exist);
* the known theory constants of the reference.
"""
import math
import os
from fractions import Fraction

import numpy as np
import pytest

from conftest import GOLDEN, boxes_from_hex, box_from_hex
from circlecover_gb300 import workloads as W
from oracle import oracle as O

SPECIALS = np.array([0.0, -0.0, 1.0, -1.0, 0.5, 2.0, 3.0, 0.1, 1e-300, -1e-300, 5e-324, -5e-324, 2.2250738585072014e-308,
                     1.7976931348623157e308, -1.7976931348623157e308, np.inf, -np.inf, np.nan, 1e300, 1e-160, 7.0,
                     0.61, 9.0 / 64.0, 1.0 + 2 ** -52, 1.0 - 2 ** -53])


def operands(n, seed):
    rng = np.random.default_rng(seed)
    a = rng.standard_normal(n) * np.exp2(rng.integers(-60, 60, n))
    b = rng.standard_normal(n) * np.exp2(rng.integers(-60, 60, n))
    wide_a = np.ldexp(rng.random(n // 8) + 0.5, rng.integers(-1074, 1023, n // 8))
    wide_b = np.ldexp(rng.random(n // 8) + 0.5, rng.integers(-1074, 1023, n // 8))
    sa, sb = np.meshgrid(SPECIALS, SPECIALS)
    a = np.concatenate([a, wide_a, -wide_a, sa.ravel(), a[: n // 8]])
    b = np.concatenate([b, wide_b, wide_b, sb.ravel(), -a[: n // 8] * (1 + 2 ** -52)])
    return a, b


def fma(a, b, c):
    """a*b+c rounded once (exact rational arithmetic; float() of a Fraction
    rounds to nearest)."""
    return float(Fraction(a) * Fraction(b) + Fraction(c))


def same_bits(x, y):
    return np.array_equal(x.view(np.uint64), y.view(np.uint64)) or bool(
        np.all((x.view(np.uint64) == y.view(np.uint64)) | (np.isnan(x) & np.isnan(y))))


@pytest.mark.parametrize("op", [0, 1, 2, 3, 4])
@pytest.mark.parametrize("up", [False, True])
def test_rounding_layer_matches_fenv(port, op, up):
    a, b = operands(200_000, 7 + op)
    if op >= 3:
        a = np.abs(a) if op == 3 else a
        b = None
    fast = port.round(op, up, a, b)
    exact = port.round(op, up, a, b, exact_fenv=True)
    assert same_bits(fast, exact)


def test_subinterval_covers_and_ends_exactly(port):
    rng = np.random.default_rng(3)
    for _ in range(2000):
        lo = rng.random() * 3
        hi = lo + rng.random() * 2
        n = int(rng.integers(1, 300))
        prev_hi = None
        for i in range(n):
            l, u = port.subinterval(lo, hi, i, n)
            if i == 0:
                assert l == lo
            assert l <= u
            if prev_hi is not None:
                assert l == prev_hi  # consecutive pieces share the FMA-computed point
            prev_hi = u
        assert prev_hi == hi


def test_subinterval_is_fma_form(port):
    rng = np.random.default_rng(4)
    for _ in range(20000):
        lo = rng.random() * 3
        hi = lo + rng.random() * 2
        n = int(rng.integers(2, 300))
        i = int(rng.integers(0, n - 1))
        diff = (hi - lo) / n
        l, u = port.subinterval(lo, hi, i, n)
        assert l == fma(diff, float(i), lo)
        assert u == fma(diff, float(i + 1), lo)


def test_port_matches_golden_eval(port, golden_eval):
    boxes, masks, ops, parts = golden_eval
    got = port.tight_eval(boxes, threads=4)
    bad = np.nonzero(got != masks)[0]
    assert len(bad) == 0, "mismatching boxes: %s" % bad[:10]


def test_golden_eval_exercises_every_bit(golden_eval):
    boxes, masks, ops, parts = golden_eval
    for bit in range(7):
        assert ((masks >> bit) & 1).sum() > 0, bit
    assert ((masks >> bit) & 1).sum() < len(masks)


def test_workload_generator_reproduces_golden_boxes(golden_eval):
    boxes, masks, ops, parts = golden_eval
    regen = np.concatenate([W.tight_microbench(int(parts[0]), seed=1), W.tight_near_critical(int(parts[1]), seed=5)])
    n = len(regen)
    assert np.array_equal(regen.view(np.uint64), boxes[:n].view(np.uint64))


def test_op_counts_port_equal_reference_counts(port_count, golden_eval):
    """The algorithmic work per box (directed-rounding primitives executed by
    the reference's code) bounds the port's: the port hoists invariant
    constants, so it never executes more operations."""
    boxes, masks, ops, parts = golden_eval
    got, port_ops = port_count.tight_eval(boxes[:2000], threads=1, count_ops=True)
    assert np.all(port_ops <= ops[:2000])
    assert port_ops.sum() > 0


@pytest.mark.parametrize("case", range(4))
def test_port_matches_golden_proofs(port, golden_prove, case):
    c = golden_prove[case]
    g = O.make_grid(c["la_init"], c["r_init"], c["gens"], c["r_gen"])
    crit, st = port.tight_prove(box_from_hex(c["root"]), g, threads=4)
    want = boxes_from_hex(c["criticals"])
    assert len(crit) == len(want)
    assert np.array_equal(crit.view(np.uint64), want.view(np.uint64))
    assert st["digest"] == c["stats"]["digest"]
    assert st["counts"] == c["stats"]["counts"]
    assert st["gen_sizes"] == c["stats"]["gen_sizes"]
    assert st["leaf_evals"] == c["stats"]["leaf_evals"]


def test_port_matches_reference_live_random(ref, port):
    for seed, gen in [(11, W.tight_microbench), (12, W.tight_near_critical)]:
        boxes = gen(60_000, seed=seed)
        a = ref.tight_eval(boxes, threads=8)
        b = port.tight_eval(boxes, threads=8)
        assert np.array_equal(a, b)


def test_port_matches_reference_live_proof(ref, port):
    root = W.tight_root(1.2, 1.25)
    g = O.make_grid(3, (16, 16, 16, 16), (2, 1), (16, 16, 8, 8))
    ca, sa = ref.tight_prove(root, g, threads=8)
    cb, sb = port.tight_prove(root, g, threads=8)
    assert np.array_equal(ca.view(np.uint64), cb.view(np.uint64))
    assert sa == sb


def test_theory_constants(ref):
    # critical ratio at lambda = 1 is 195/256 (rectangle_size_bound/can_recurse.cu:27)
    lo_hi = __import__("ctypes").c_double()
    lo = ref.lib.ccref_tight_critical_ratio(1.0, 1.0, lo_hi)
    assert lo <= 195 / 256 <= lo_hi.value
    # break-even lambda_2 = sqrt(sqrt(7)/2 - 1/4): both formulas agree there
    l2 = W.LAMBDA_2
    three = (3 / 256) / l2 * (16 * l2 * l2 + 40 + 9 / (l2 * l2))
    two = l2 / 4 + 1 / (2 * l2)
    assert abs(three - two) < 1e-12


def test_prepared_leaf_form_equals_plain(port):
    """The proof's leaf form of r1_r2_r3_strategies prepared once per r3 cell
    (leaf123_prepare / leaf123_check) gives the criterion's result and trap
    status for every upper bound of r4 below r3."""
    import ctypes
    lib = port.lib
    lib.ccport_leafprep_mismatches.argtypes = [ctypes.c_void_p, ctypes.c_size_t, ctypes.c_int]
    lib.ccport_leafprep_mismatches.restype = ctypes.c_size_t
    for gen, seed in [(W.tight_microbench, 64), (W.tight_near_critical, 65)]:
        boxes = np.ascontiguousarray(gen(20000, seed=seed))
        assert lib.ccport_leafprep_mismatches(boxes.ctypes.data, len(boxes), 9) == 0
    root = W.tight_root(1.0, 1.02)
    g = O.make_grid(2, (8, 8, 8, 8), (), (8, 8, 8, 8))
    crit, st = port.tight_prove(root, g, threads=4)
    edge = np.ascontiguousarray(np.concatenate([crit, W.tight_near_critical(5000, seed=66)]))
    assert lib.ccport_leafprep_mismatches(edge.ctypes.data, len(edge), 17) == 0
    # the golden boxes: microbench, near-critical and the hand-made edge cases
    # (point intervals, lambda = 1 and the break-even, empty and subnormal radii)
    z = np.load(os.path.join(GOLDEN, "tight_eval_golden.npz"))
    gold = np.ascontiguousarray(z["boxes"]).view(W.TIGHT_BOX).reshape(-1)
    assert lib.ccport_leafprep_mismatches(gold.ctypes.data, len(gold), 9) == 0
    lib.ccport_resume_mismatches.argtypes = [ctypes.c_void_p, ctypes.c_size_t]
    lib.ccport_resume_mismatches.restype = ctypes.c_size_t
    assert lib.ccport_resume_mismatches(gold.ctypes.data, len(gold)) == 0


def test_strip_bisection_resumes_exactly(port):
    """The strip-width bisection resumed from its bracket and step count after
    any number of steps (how the evaluation's second strip-width kernel
    continues the jobs the first stopped) ends with the same width and trap
    status as the bisection run in one go."""
    import ctypes
    lib = port.lib
    lib.ccport_resume_mismatches.argtypes = [ctypes.c_void_p, ctypes.c_size_t]
    lib.ccport_resume_mismatches.restype = ctypes.c_size_t
    for gen, seed in [(W.tight_microbench, 67), (W.tight_near_critical, 68)]:
        boxes = np.ascontiguousarray(gen(20000, seed=seed))
        assert lib.ccport_resume_mismatches(boxes.ctypes.data, len(boxes)) == 0


def test_prepared_criteria_equal_plain(port):
    """The proof engine's hoisted criteria (prepare once per parent cell, check
    per child bound) agree with the plain criteria for every bound."""
    import ctypes
    lib = port.lib
    lib.ccport_prepared_mismatches.argtypes = [ctypes.c_void_p, ctypes.c_size_t, ctypes.c_int]
    lib.ccport_prepared_mismatches.restype = ctypes.c_size_t
    for gen, seed in [(W.tight_microbench, 61), (W.tight_near_critical, 62)]:
        boxes = np.ascontiguousarray(gen(20000, seed=seed))
        assert lib.ccport_prepared_mismatches(boxes.ctypes.data, len(boxes), 9) == 0
    # boxes from the proof's own grid near lambda = 1 (where most strategies are close calls)
    root = W.tight_root(1.0, 1.02)
    g = O.make_grid(2, (8, 8, 8, 8), (), (8, 8, 8, 8))
    crit, st = port.tight_prove(root, g, threads=4)
    edge = np.ascontiguousarray(np.concatenate([crit, W.tight_near_critical(5000, seed=63)]))
    assert lib.ccport_prepared_mismatches(edge.ctypes.data, len(edge), 17) == 0
