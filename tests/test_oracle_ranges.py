"""CPU tier: the oracle's task-range generations (the unit of the sampled
parity fixtures of the full-size proofs) agree with its whole-proof entry
points, and the port agrees with the reference's own criteria on them."""
import numpy as np
import pytest

import circlecover_gb300 as cg
from circlecover_gb300 import workloads as W
from oracle import oracle as O


@pytest.fixture(scope="module")
def ref():
    O.ensure_built()
    if not O.ref_available():
        pytest.skip("reference sources not available")
    return O.Ref()


def test_sb_generation_ranges_add_up_to_the_initial_pass(ref, port):
    root = W.sb_root(1.0, 1.05)
    rs = (4, 4, 4, 4, 4, 4)
    whole, wflags, wst = ref.sb_prove(root, cg.make_sb_grid(2, rs, gens=0), threads=4)
    c, f, st = ref.sb_generation(np.array([root]), 0, 2, rs, 0, 2 * 16, threads=4)
    assert np.array_equal(c.view(np.uint64), whole.view(np.uint64)) and np.array_equal(f, wflags)
    assert st["digest"] == wst["digest"] and st["leaf_evals"] == wst["leaf_evals"]
    parts = [ref.sb_generation(np.array([root]), 0, 2, rs, lo, lo + 8, threads=2)[2] for lo in range(0, 32, 8)]
    assert sum(p["digest"] for p in parts) % (1 << 64) == wst["digest"]
    assert sum(p["leaf_evals"] for p in parts) == wst["leaf_evals"]
    for lo in (0, 5, 17):
        a = ref.sb_generation(np.array([root]), 0, 2, rs, lo, lo + 3, threads=2)
        b = port.sb_generation(np.array([root]), 0, 2, rs, lo, lo + 3, threads=2)
        assert np.array_equal(a[0].view(np.uint64), b[0].view(np.uint64)) and a[2]["digest"] == b[2]["digest"]


def test_tight_generation_of_the_reference_equals_the_port(ref, port):
    root = W.tight_root(1.0, 1.05)
    for lo, hi in ((0, 2), (3, 4)):
        a = ref.tight_generation(np.array([root]), 4, (8, 8, 8, 8), lo, hi, threads=2)
        b = port.tight_generation(np.array([root]), 4, (8, 8, 8, 8), lo, hi, threads=2)
        assert np.array_equal(a[0].view(np.uint64), b[0].view(np.uint64))
        assert a[1]["digest"] == b[1]["digest"] and a[1]["counts"] == b[1]["counts"]
