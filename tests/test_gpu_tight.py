"""GPU tier: the CUDA prover through its C ABI against the oracle.

Bit-exact everywhere (integer verdict masks, FP64 interval endpoints):
* the device directed-rounding primitives equal the host rounding layer;
* nvcc's default contraction of the reference's split expression equals the
  explicit FMA the prover uses;
* cc_tight_eval / cc_tight_eval_device verdict masks equal the golden
  fixtures (made by the reference's code) and the CPU port on larger sets;
* cc_tight_prove critical boxes, trace digest and per-outcome counts equal the
  golden proofs and the CPU port.
"""
import ctypes

import numpy as np
import pytest

from conftest import box_from_hex, boxes_from_hex
from circlecover_gb300 import workloads as W
import circlecover_gb300 as cg
from oracle import oracle as O
from test_oracle import operands, same_bits

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("op", [0, 1, 2, 3, 4])
@pytest.mark.parametrize("up", [False, True])
def test_device_rounding_equals_host_layer(prover, port, op, up):
    a, b = operands(400_000, 100 + op)
    if op >= 3:
        a = np.abs(a) if op == 3 else a
        b = None
    dev = prover.selftest_round(op, up, a, b)
    host = port.round(op, up, a, b, exact_fenv=True)
    assert same_bits(dev, host)


def test_nvcc_contracts_split_expression_to_fma(prover):
    rng = np.random.default_rng(9)
    n = 200_000
    lo = rng.random(n) * 3
    hi = lo + rng.random(n) * np.exp2(rng.integers(-30, 2, n))
    cnt = rng.integers(1, 300, n).astype(np.int32)
    idx = (rng.random(n) * cnt).astype(np.int32)
    explicit, plain = prover.selftest_subinterval(lo, hi, idx, cnt)
    assert np.array_equal(explicit.view(np.uint64), plain.view(np.uint64))


def test_eval_matches_golden(prover, golden_eval):
    boxes, masks, ops, parts = golden_eval
    got = prover.tight_eval(boxes)
    bad = np.nonzero(got != masks)[0]
    assert len(bad) == 0, "mismatching boxes %s" % bad[:10]
    assert prover.last_launch_count >= 1


def test_eval_matches_port_large(prover, port):
    for seed, gen, n in [(21, W.tight_microbench, 1 << 18), (22, W.tight_near_critical, 1 << 17)]:
        boxes = gen(n, seed=seed)
        assert np.array_equal(prover.tight_eval(boxes), port.tight_eval(boxes, threads=16))


def test_eval_device_soa(prover, port):
    import torch
    boxes = W.tight_microbench(50_000, seed=31)
    soa = torch.from_numpy(W.to_soa(boxes)).cuda()
    masks = torch.zeros(len(boxes), dtype=torch.int32, device="cuda")
    prover.tight_eval_device(soa.data_ptr(), len(boxes), masks.data_ptr())
    # the entry point runs on the handle's stream; wait for the device
    torch.cuda.synchronize()
    cc_stream_sync(prover)
    got = masks.cpu().numpy().view(np.uint32)
    assert np.array_equal(got, port.tight_eval(boxes, threads=16))


def test_stage_timing_times_three_kernels_without_changing_masks(prover, port):
    import torch
    boxes = W.tight_microbench(40_000, seed=32)
    soa = torch.from_numpy(W.to_soa(boxes)).cuda()
    masks = torch.zeros(len(boxes), dtype=torch.int32, device="cuda")
    torch.cuda.synchronize()
    with pytest.raises(Exception):
        prover.stage_times()  # nothing timed yet
    prover.set_stage_timing(True)
    prover.tight_eval_device(soa.data_ptr(), len(boxes), masks.data_ptr())
    ms = prover.stage_times()
    prover.set_stage_timing(False)
    assert len(ms) == 3 and all(t > 0 for t in ms)
    assert np.array_equal(masks.cpu().numpy().view(np.uint32), port.tight_eval(boxes, threads=16))


def cc_stream_sync(prover):
    import torch
    torch.cuda.synchronize()
    # a zero-box call is a no-op; a small host call drains the handle's stream
    prover.tight_eval(W.tight_microbench(1, seed=0))


def test_eval_empty_and_ragged(prover, port):
    assert len(prover.tight_eval(np.zeros(0, dtype=W.TIGHT_BOX))) == 0
    for n in [1, 31, 33, 127, 129, 1000]:
        boxes = W.tight_microbench(n, seed=40 + n)
        assert np.array_equal(prover.tight_eval(boxes), port.tight_eval(boxes))


@pytest.mark.parametrize("plain", [False, True])
@pytest.mark.parametrize("case", range(4))
def test_prove_matches_golden(prover, golden_prove, case, plain):
    c = golden_prove[case]
    g = cg.make_grid(c["la_init"], c["r_init"], c["gens"], c["r_gen"])
    crit, st = prover.tight_find_critical_intervals(box_from_hex(c["root"]), g, plain=plain)
    want = boxes_from_hex(c["criticals"])
    assert len(crit) == len(want)
    assert np.array_equal(crit.view(np.uint64), want.view(np.uint64))
    assert st["digest"] == c["stats"]["digest"]
    assert st["counts"] == c["stats"]["counts"]
    assert st["gen_sizes"] == c["stats"]["gen_sizes"]
    assert st["leaf_evals"] == c["stats"]["leaf_evals"]
    assert st["kernel_launches"] > 0


@pytest.mark.parametrize("la", [(1.0, 1.0 + 0.1 / 64), (1.03, 1.04), (1.6, 1.62)])
def test_prove_matches_port_bigger(prover, port, la):
    root = W.tight_root(*la)
    gg = dict(la_init=2, r_init=(32, 64, 32, 32), gens=(1, 2), r_gen=(32, 32, 32, 16))
    pc, ps = port.tight_prove(root, O.make_grid(**gg), threads=16)
    for plain in (False, True):
        crit, st = prover.tight_find_critical_intervals(root, cg.make_grid(**gg), plain=plain)
        assert np.array_equal(crit.view(np.uint64), pc.view(np.uint64))
        for k in ("digest", "counts", "gen_sizes", "leaf_evals"):
            assert st[k] == ps[k], k


def test_prove_rejects_bad_grid(prover):
    root = W.tight_root(1.0, 1.1)
    with pytest.raises(cg.CudaError):
        prover.tight_find_critical_intervals(root, cg.make_grid(0, (8, 8, 8, 8)))
    with pytest.raises(cg.CudaError):
        prover.tight_find_critical_intervals(root, cg.make_grid(2, (8, 8, 4096, 8)))


def test_prove_empty_root(prover):
    # lambda range whose r1 range does not meet the root's r1 interval
    root = W.tight_root(1.0, 1.01)
    root["r"][0] = (5.0, 6.0)
    crit, st = prover.tight_find_critical_intervals(root, cg.make_grid(2, (8, 8, 8, 8), (1,)))
    assert len(crit) == 0
    assert st["leaf_evals"] == 0


def test_autotuned_passes_give_the_same_masks(prover, port):
    import torch
    boxes = W.tight_microbench(1 << 16, seed=44)
    soa = torch.from_numpy(W.to_soa(boxes)).cuda()
    masks = torch.zeros(len(boxes), dtype=torch.int32, device="cuda")
    torch.cuda.synchronize()
    rep = prover.autotune_eval(soa.data_ptr(), len(boxes), masks.data_ptr())
    assert set(rep) == {"k_eval_main", "k_eval_cover", "k_eval_gaps"}
    for r in rep.values():
        assert r["min_blocks"] in (1, 4, 8) and r["blocks_per_sm"] in (2, 4, 8, 16)
        assert r["ms"] <= r["ms_default"] * 1.0001
    got = prover.tight_eval(boxes)  # runs with the tuned settings
    assert np.array_equal(got, port.tight_eval(boxes, threads=16))


def test_checkpoint_resume_equals_uninterrupted_run(prover, golden_prove, tmp_path):
    c = golden_prove[3]  # three refinement generations
    full = cg.make_grid(c["la_init"], c["r_init"], c["gens"], c["r_gen"])
    first = cg.make_grid(c["la_init"], c["r_init"], c["gens"][:1], c["r_gen"])
    path = str(tmp_path / "tight.ckpt")
    prover.set_checkpoint(path)
    try:
        prover.tight_find_critical_intervals(box_from_hex(c["root"]), first)  # init + generation 1
    finally:
        prover.set_checkpoint(None)
    crit, st = prover.tight_resume(path, full)
    want = boxes_from_hex(c["criticals"])
    assert np.array_equal(crit.view(np.uint64), want.view(np.uint64))
    for k in ("digest", "counts", "gen_sizes", "leaf_evals"):
        assert st[k] == c["stats"][k], k
    with pytest.raises(cg.CudaError):  # a schedule that does not extend the checkpoint's
        prover.tight_resume(path, cg.make_grid(c["la_init"] * 2, c["r_init"], c["gens"], c["r_gen"]))
