import json
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def port():
    from oracle import oracle as O
    O.ensure_built()
    return O.Port()


@pytest.fixture(scope="session")
def port_count():
    from oracle import oracle as O
    O.ensure_built()
    return O.Port(count=True)


@pytest.fixture(scope="session")
def ref():
    from oracle import oracle as O
    O.ensure_built()
    if not O.ref_available():
        pytest.skip("reference sources not present: oracle/_ref not built")
    return O.Ref()


@pytest.fixture(scope="session")
def golden_eval():
    from circlecover_gb300 import workloads as W
    z = np.load(os.path.join(GOLDEN, "tight_eval_golden.npz"))
    boxes = np.ascontiguousarray(z["boxes"]).view(W.TIGHT_BOX).reshape(-1)
    return boxes, z["masks"], z["ops"], z["parts"]


@pytest.fixture(scope="session")
def golden_prove():
    with open(os.path.join(GOLDEN, "tight_prove_golden.json")) as f:
        return json.load(f)["cases"]


@pytest.fixture(scope="session")
def lib_path():
    from circlecover_gb300 import _build
    return _build.build()


@pytest.fixture(scope="session")
def prover(lib_path):
    import circlecover_gb300 as cg
    p = cg.Prover(0)
    yield p
    p.close()


def box_from_hex(h):
    from circlecover_gb300 import workloads as W
    b = np.zeros(1, dtype=W.TIGHT_BOX)
    b["la"][0] = (float.fromhex(h[0][0]), float.fromhex(h[0][1]))
    for k in range(4):
        b["r"][0, k] = (float.fromhex(h[k + 1][0]), float.fromhex(h[k + 1][1]))
    return b[0]


def boxes_from_hex(rows):
    from circlecover_gb300 import workloads as W
    if not rows:
        return np.zeros(0, dtype=W.TIGHT_BOX)
    return np.array([box_from_hex(r) for r in rows], dtype=W.TIGHT_BOX)
