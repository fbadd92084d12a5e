"""GPU tier: FP64 certification of the FP32 pre-filter's verdicts.

The evaluation and the proofs decide most criteria on outward-rounded FP32
enclosures of the FP64 values.  Every "true" they decide is checked again in
FP64 directed rounding before it counts (include/circlecover_gb300.h,
cc_set_eval_certify; cc_prove_stats.fp32_first).  These tests show

* the certifier itself cannot be fooled: run with any call number, it never
  accepts a criterion that the oracle's FP64 evaluation rejects, and with
  every call evaluated it is the FP64 criterion;
* certification changes no verdict (masks with and without it, and the
  oracle's, are equal bit for bit) and none of its checks fails;
* the proofs' certified leaf criteria leave criticals, trace and counts as
  the oracle has them.
"""
import numpy as np
import pytest

import circlecover_gb300 as cg
from circlecover_gb300 import workloads as W
from oracle import oracle as O

pytestmark = pytest.mark.gpu

# record groups of the certifier and their verdict bits (CC_TV_*)
GROUP_BITS = {0: 0, 1: 1, 2: 3, 3: 4}


def _boxes():
    return np.concatenate([W.tight_microbench(40_000, seed=301), W.tight_near_critical(40_000, seed=302)])


@pytest.mark.parametrize("group", [0, 1, 2, 3])
def test_certifier_never_accepts_a_false_criterion(prover, port, group):
    boxes = _boxes()
    masks = port.tight_eval(boxes, threads=16)
    boxes = boxes[(masks >> 31) == 0]  # boxes on which no criterion reaches a trap site
    masks = masks[(masks >> 31) == 0]
    truth = ((masks >> GROUP_BITS[group]) & 1).astype(bool)
    n = len(boxes)
    assert truth.any() and not truth.all()
    # every call evaluated: the FP64 criterion itself
    full = prover.selftest_certify(group, boxes, np.full(n, -1))
    assert np.array_equal(full, truth)
    accepted_any = np.zeros(n, dtype=bool)
    record_any = np.zeros(n, dtype=bool)
    for call in range(0, 6):
        got = prover.selftest_certify(group, boxes, np.full(n, call))
        # one call evaluated, the others forced to "false": never a false accept
        assert not (got & ~truth).any(), (group, call, np.nonzero(got & ~truth)[0][:8])
        accepted_any |= got
        # the record form (the call evaluated afterwards on its stored
        # arguments) accepts no more than the direct form
        rec = prover.selftest_certify(group, boxes, np.full(n, call), record=True)
        assert not (rec & ~got).any(), (group, call, np.nonzero(rec & ~got)[0][:8])
        record_any |= rec
    # and every true criterion is accepted with some call number, in both forms
    assert np.array_equal(accepted_any, truth)
    assert np.array_equal(record_any, truth)


def test_certified_masks_equal_uncertified_and_oracle(port):
    import torch
    boxes = np.concatenate([W.tight_microbench(1 << 17, seed=311), W.tight_near_critical(1 << 16, seed=312)])
    want = port.tight_eval(boxes, threads=16)
    soa = torch.from_numpy(W.to_soa(boxes)).cuda()
    out = torch.zeros(len(boxes), dtype=torch.int32, device="cuda")
    p = cg.Prover(0)
    try:
        got = {}
        for certify in (True, False):
            p.set_eval_certify(certify)
            out.zero_()
            torch.cuda.synchronize()
            p.tight_eval_device(soa.data_ptr(), len(boxes), out.data_ptr())
            torch.cuda.synchronize()
            got[certify] = out.cpu().numpy().view(np.uint32).copy()
            c = p.eval_cert_counts()
            if certify:
                assert c["failed"] == 0, c
                # every FP32-decided true verdict of the record groups was certified
                fp32_boxes = len(boxes) - p.eval_counts()["fp64_boxes"]
                assert 0 < c["r1"] <= fp32_boxes
                assert c["cover"] > 0 and c["gaps"] > 0
            else:
                assert sum(c.values()) == 0, c
        assert np.array_equal(got[True], want)
        assert np.array_equal(got[False], want)
        # the host entry point certifies too
        p.set_eval_certify(True)
        assert np.array_equal(p.tight_eval(boxes[:50_000]), want[:50_000])
    finally:
        p.close()


def test_certified_eval_of_adversarial_boxes(prover, port):
    from test_gpu_tight import _adversarial_boxes
    boxes = _adversarial_boxes(1 << 15, 313)
    assert np.array_equal(prover.tight_eval(boxes), port.tight_eval(boxes, threads=16))


@pytest.mark.parametrize("learned", [False, True])
def test_proof_certification_counts(prover, port, learned):
    root = W.tight_root(1.0, 1.02)
    grid = cg.make_grid(8, (16, 32, 32, 32), gens=(1,), r_gen=(16, 16, 16, 16))
    if learned:
        prover.mlp_init(11)
    crit, st = prover.tight_find_critical_intervals(root, grid, learned=learned)
    pc, ps = port.tight_prove(root, O.make_grid(8, (16, 32, 32, 32), gens=(1,), r_gen=(16, 16, 16, 16)), threads=16)
    assert np.array_equal(crit.view(np.uint64), pc.view(np.uint64))
    assert st["gen_sizes"] == ps["gen_sizes"] and st["leaf_evals"] == ps["leaf_evals"]
    if not learned:
        assert st["digest"] == ps["digest"]
    assert st["cert_failures"] == 0
    assert st["fp32_first"][3] == 0
    assert st["fp32_first"][2] > 0  # FP32 "true" leaf verdicts, each certified in FP64
