"""Size-bound criteria (rectangle_size_bound): the CPU port against the
reference's own code (golden fixtures always, the live reference library
where it exists), the hoisted constants against their formulas, and the GPU
evaluator against both."""
import ctypes
import os

import numpy as np
import pytest

from conftest import GOLDEN
from circlecover_gb300 import workloads as W


@pytest.fixture(scope="module")
def sb_golden():
    z = np.load(os.path.join(GOLDEN, "sb_eval_golden.npz"))
    boxes = np.ascontiguousarray(z["boxes"]).view(W.SB_BOX).reshape(-1)
    return boxes, z["masks"], z["parts"]


def test_port_matches_golden(port, sb_golden):
    boxes, masks, parts = sb_golden
    got = port.sb_eval(boxes, threads=8)
    bad = np.nonzero(got != masks)[0]
    assert len(bad) == 0, "mismatching boxes %s" % bad[:10]


def test_golden_exercises_every_criterion(sb_golden):
    boxes, masks, parts = sb_golden
    for bit in list(range(15)) + list(range(15, 20)):
        assert ((masks >> bit) & 1).sum() > 0, bit
    assert ((masks >> 31) & 1).sum() > 0  # some boxes reach a trap site


def test_generator_reproduces_golden_boxes(sb_golden):
    boxes, masks, parts = sb_golden
    regen = np.concatenate([W.sb_boxes(int(parts[0]), seed=3, la_hi=2.5), W.sb_boxes(int(parts[1]), seed=4, la_hi=8.0)])
    assert np.array_equal(regen.view(np.uint64), boxes[: len(regen)].view(np.uint64))


def test_constants_equal_their_formulas(port):
    lib = port.lib
    lib.ccport_sb_constants.argtypes = [ctypes.c_void_p]
    out = np.zeros(7)
    lib.ccport_sb_constants(out.ctypes.data)
    # the hex literals in cc_sb.cuh / cc_tight.cuh
    want = [float.fromhex(h) for h in ("0x1.505ca676dd495p-6", "0x1.984097fce8a6cp-1", "0x1.9efda00c5d64cp-3",
                                       "0x1.4586fa613f21cp-1", "0x1.4586fa613f222p-1", "0x1.0929ffddd109ap+0",
                                       "0x1.0929ffddd109bp+0")]
    assert [float(x).hex() for x in out] == [float(x).hex() for x in want]


def test_port_matches_reference_live(ref, port):
    for seed, la_hi in [(31, 2.5), (32, 8.0), (33, 1.2)]:
        boxes = W.sb_boxes(6000, seed=seed, la_hi=la_hi)
        assert np.array_equal(ref.sb_eval(boxes, threads=8), port.sb_eval(boxes, threads=8))


@pytest.mark.gpu
def test_gpu_sb_eval_matches_golden(prover, sb_golden):
    boxes, masks, parts = sb_golden
    got = prover.sb_eval(boxes)
    bad = np.nonzero(got != masks)[0]
    assert len(bad) == 0, "mismatching boxes %s" % bad[:10]


@pytest.mark.gpu
def test_gpu_sb_eval_matches_port(prover, port):
    for seed, la_hi, n in [(41, 2.5, 30000), (42, 8.0, 20000)]:
        boxes = W.sb_boxes(n, seed=seed, la_hi=la_hi)
        assert np.array_equal(prover.sb_eval(boxes), port.sb_eval(boxes, threads=16))


@pytest.mark.gpu
def test_gpu_sb_eval_device_soa(prover, port):
    import torch
    boxes = W.sb_boxes(5000, seed=43)
    soa = torch.from_numpy(W.to_soa(boxes)).cuda()
    masks = torch.zeros(len(boxes), dtype=torch.int32, device="cuda")
    torch.cuda.synchronize()
    prover.sb_eval_device(soa.data_ptr(), len(boxes), masks.data_ptr())
    prover.sb_eval(boxes[:1])  # drains the handle's stream
    torch.cuda.synchronize()
    assert np.array_equal(masks.cpu().numpy().view(np.uint32), port.sb_eval(boxes, threads=16))
