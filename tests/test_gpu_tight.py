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
import os

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


def test_eval_whole_microbench_matches_port(prover, port):
    """Config 2 at its full size: all 2^24 boxes of the bench workload (seed
    1), certified masks from the device entry point equal the port's (all
    host threads, about half a minute)."""
    import torch
    n = 1 << 24
    boxes = W.tight_microbench(n, seed=1)
    soa = torch.from_numpy(W.to_soa(boxes)).cuda()
    masks = torch.empty(n, dtype=torch.int32, device="cuda")
    torch.cuda.synchronize()
    prover.tight_eval_device(soa.data_ptr(), n, masks.data_ptr())
    torch.cuda.synchronize()
    got = masks.cpu().numpy().view(np.uint32)
    del soa, masks
    want = port.tight_eval(boxes, threads=os.cpu_count() or 16)
    assert np.array_equal(got, want), int((got != want).sum())


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


def test_stage_timing_times_the_passes_without_changing_masks(prover, port):
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
    # six passes: FP32, FP64, the two bisections, certification, repair
    assert len(ms) == 6 and all(t > 0 for t in ms[:5]) and ms[5] >= 0
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
    assert set(rep) == {"k_eval_f32", "k_eval_main", "k_eval_cover", "k_eval_gaps"}
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


def _bisection_rows(prover, which, rows, lo, hi, rounds=2200):
    """Runs the bisection of every row to its FP64 fixpoint on the host,
    each step decided by the device's FP64 predicate; checks every step the
    FP32 enclosure of the step's point decides against it.  Returns (steps,
    FP32-decided steps, final lo per row)."""
    steps = decided = 0
    for _ in range(rounds):
        mid = 0.5 * (lo + hi)
        act = (mid > lo) & (mid < hi)
        if not act.any():
            break
        args = rows[act].copy()
        args[:, 6] = args[:, 7] = mid[act]
        f32, f64 = prover.selftest_bisection_f32(which, args)
        assert not (f64 & 2).any()  # no trap site on these inputs
        ok = f32 >= 0
        assert np.array_equal(f32[ok], f64[ok] & 1), "an FP32 decision differs from the FP64 predicate"
        steps += int(act.sum())
        decided += int(ok.sum())
        yes = np.zeros(len(rows), dtype=bool)
        yes[np.nonzero(act)[0]] = (f64 & 1) == 1
        lo = np.where(act & yes, mid, lo)
        hi = np.where(act & ~yes, mid, hi)
    return steps, decided, lo


def _check_ranges(prover, which, rows, lo, hi, points=33):
    """FP32 decisions over whole ranges [lo, hi]: where one is made, the FP64
    predicate has that outcome at points spread over the range and at its
    ends.  Returns how many ranges were decided."""
    args = rows.copy()
    args[:, 6], args[:, 7] = lo, hi
    f32, _ = prover.selftest_bisection_f32(which, args)
    dec = f32 >= 0
    if not dec.any():
        return 0
    sub = args[dec]
    for k in range(points):
        t = args.copy()[dec]
        t[:, 6] = sub[:, 6] + (sub[:, 7] - sub[:, 6]) * (k / (points - 1))
        t[:, 6] = np.minimum(np.maximum(t[:, 6], sub[:, 6]), sub[:, 7])
        t[:, 7] = t[:, 6]
        _, f64 = prover.selftest_bisection_f32(which, t)
        assert np.array_equal(f64 & 1, f32[dec]), "a whole-range FP32 decision differs from the FP64 predicate"
    return int(dec.sum())


def _gaps_rows(n, seed):
    b = W.tight_microbench(n, seed=seed)
    r = b["r"][:, :, 0].copy()
    r[:, 2] = np.maximum(r[:, 2], r[:, 3])
    r[:, 1] = np.maximum(r[:, 1], r[:, 2])
    r[:, 0] = np.maximum(r[:, 0], r[:, 1])
    keep = (4 * r[:, 0] - 1 > 0) & (4 * r[:, 1] - 1 > 0)
    r = r[keep]
    rows = np.zeros((len(r), 8))
    rows[:, 0], rows[:, 1] = r[:, 0], r[:, 1]
    rows[:, 2], rows[:, 3] = np.sqrt(4 * r[:, 0] - 1), np.sqrt(4 * r[:, 1] - 1)
    rows[:, 4] = r[:, 3]
    return rows


def _cover_rows(prover, n, seed):
    b = W.tight_microbench(n, seed=seed)
    rows = np.zeros((len(b), 8))
    rows[:, :3] = b["r"][:, :3, 0]
    rows[:, 6] = rows[:, 7] = 0.3
    _, f64 = prover.selftest_bisection_f32(0, rows)
    keep = (f64 & 1) == 1  # the boxes whose strip of width 0.3 is realizable
    return rows[keep], b["la"][keep, 1].copy()


@pytest.mark.parametrize("which", [0, 1])
def test_fp32_bisection_decisions_equal_fp64(prover, which):
    """The FP32 enclosures that decide bisection steps, and whole ranges of
    steps, before the FP64 predicate runs never contradict it: along the
    bisection paths of microbench boxes to their fixpoints, at points
    scattered around each fixpoint, and over the starting ranges and ranges
    around the fixpoints.  The device's whole bisection (shortcuts included)
    returns the host-driven FP64 bisection's result bit for bit."""
    if which == 1:
        rows = _gaps_rows(1 << 14, seed=61)
        lo0, hi0 = np.zeros(len(rows)), np.sqrt(rows[:, 0]) + np.sqrt(rows[:, 1])
    else:
        rows, la = _cover_rows(prover, 1 << 15, seed=62)
        lo0, hi0 = np.full(len(rows), 0.3), la
    steps, decided, fix = _bisection_rows(prover, which, rows, lo0.copy(), hi0.copy())
    assert steps > 0 and decided >= 0.25 * steps, (steps, decided)
    rng = np.random.default_rng(63 + which)
    for scale in [0.5, 2.0 ** -10, 2.0 ** -20, 2.0 ** -26, 2.0 ** -40]:
        args = rows.copy()
        args[:, 6] = args[:, 7] = np.maximum(fix * (1 + scale * rng.uniform(-1, 1, len(rows))), 0.0)
        f32, f64 = prover.selftest_bisection_f32(which, args)
        ok = f32 >= 0
        assert np.array_equal(f32[ok], f64[ok] & 1)
    n_dec = _check_ranges(prover, which, rows, lo0, hi0)
    for scale in [2.0 ** -4, 2.0 ** -12]:
        lo = np.maximum(fix * (1 - scale), lo0)
        hi = np.minimum(fix * (1 + scale), hi0)
        good = lo < hi
        n_dec += _check_ranges(prover, which, rows[good], lo[good], hi[good])
    assert n_dec > 0
    # the device's bisection with its shortcuts lands where the FP64 one does
    args = rows.copy()
    if which == 0:
        args[:, 6] = hi0
    got, trapped = prover.selftest_bisection_width(which, args)
    assert not trapped.any()
    assert np.array_equal(got.view(np.uint64), fix.view(np.uint64))


def _adversarial_boxes(n, seed):
    """Boxes with degenerate and extreme bounds: point intervals, empty
    intervals (lo > hi), zero and negative bounds, widths from 0 to huge,
    bounds near the float range limits, DBL_MAX, infinities and NaNs."""
    rng = np.random.default_rng(seed)
    base = W.tight_microbench(n, seed=seed)
    b = base.copy()
    flat = b.view(np.float64).reshape(n, 10)
    specials = np.array([0.0, -0.0, 1e-45, 1e-39, 1e-30, 1e30, 3.5e38, 1e300, W.DBL_MAX, np.inf, -1e-3, 0.25,
                         0.5, 1.0, 2.0, np.nan], dtype=np.float64)
    kind = rng.integers(0, 6, n)
    for col in range(10):
        pick = rng.random(n) < 0.15
        flat[pick, col] = rng.choice(specials, pick.sum())
    pt = kind == 1  # point intervals
    flat[pt, 1::2] = flat[pt, 0::2]
    sw = kind == 2  # empty intervals: bounds swapped
    flat[sw, 0::2], flat[sw, 1::2] = flat[sw, 1::2].copy(), flat[sw, 0::2].copy()
    tiny = kind == 3  # widths at the FP64 resolution
    with np.errstate(over="ignore"):
        flat[tiny, 1::2] = np.nextafter(flat[tiny, 0::2], np.inf)
    return b


def test_eval_adversarial_boxes_match_port(prover, port):
    """The FP32-first evaluation on degenerate, empty, huge, tiny, infinite
    and NaN bounds gives the port's masks bit for bit (trap bits included)."""
    for seed in (71, 72):
        boxes = _adversarial_boxes(1 << 16, seed)
        got = prover.tight_eval(boxes)
        want = port.tight_eval(boxes, threads=16)
        bad = np.nonzero(got != want)[0]
        assert len(bad) == 0, (seed, bad[:8], got[bad[:8]], want[bad[:8]])


def test_host_entry_staging_and_direct_paths_agree(port):
    """cc_tight_eval through pinned staging (CC_HOST_STAGING=1) and, where the
    device can access pageable host memory, in place, on a batch larger than
    one chunk of either path, equals the port."""
    import os
    boxes = W.tight_microbench((1 << 23) + 12345, seed=81)
    sample = np.r_[0:4096, (1 << 21) - 2048:(1 << 21) + 2048, len(boxes) - 4096:len(boxes)]
    want = port.tight_eval(boxes[sample], threads=16)
    old = os.environ.get("CC_HOST_STAGING")
    try:
        for staging in ("1", "0"):
            os.environ["CC_HOST_STAGING"] = staging
            p = cg.Prover(0)
            try:
                got = p.tight_eval(boxes)
            finally:
                p.close()
            assert np.array_equal(got[sample], want), staging
    finally:
        if old is None:
            os.environ.pop("CC_HOST_STAGING", None)
        else:
            os.environ["CC_HOST_STAGING"] = old


def test_eval_graph_replay_matches_direct_launches(port):
    """The evaluation's CUDA graph (cc_set_eval_graph): replays give the masks
    of direct launches, a call with other arguments re-captures, and small
    batches (grids cut to the batch) and the chunked host entry equal the
    port."""
    import torch
    p = cg.Prover(0)
    try:
        masks = {}
        for n, seed in ((70_000, 91), (50_000, 92)):
            boxes = W.tight_microbench(n, seed=seed)
            soa = torch.from_numpy(W.to_soa(boxes)).to("cuda")
            out = torch.zeros(n, dtype=torch.int32, device="cuda")
            p.set_eval_graph(False)
            p.tight_eval_device(soa.data_ptr(), n, out.data_ptr())
            torch.cuda.synchronize()
            direct = out.cpu().numpy().view(np.uint32).copy()
            p.set_eval_graph(True)
            for _ in range(3):
                out.zero_()
                p.tight_eval_device(soa.data_ptr(), n, out.data_ptr())
                torch.cuda.synchronize()
                assert np.array_equal(out.cpu().numpy().view(np.uint32), direct), n
            masks[n] = (boxes, direct)
        captures, replays = p.eval_graph_stats()
        assert captures == 2 and replays == 6, (captures, replays)
        boxes, direct = masks[50_000]
        sample = np.r_[0:2000, 48_000:50_000]
        assert np.array_equal(direct[sample], port.tight_eval(boxes[sample], threads=16))
        big = W.tight_microbench((1 << 22) + 777, seed=93)
        got = p.tight_eval(big)
        sample = np.r_[0:3000, len(big) - 3000:len(big)]
        assert np.array_equal(got[sample], port.tight_eval(big[sample], threads=16))
    finally:
        p.close()


def test_round_to_floats_equals_directed_conversions(prover):
    """The FP32 enclosures round doubles to floats by integer operations on
    the bits; they equal __double2float_rd / __double2float_ru bit for bit
    (random bit patterns, the normal float range, exact floats and their
    neighbours, the range boundaries, zeros, infinities, NaN)."""
    rng = np.random.default_rng(77)
    bits = rng.integers(0, 2**63, 400_000, dtype=np.int64).astype(np.uint64)
    bits[::2] |= np.uint64(1 << 63)
    pat = bits.view(np.float64)
    logu = np.exp2(rng.uniform(-135, 135, 400_000)) * rng.choice([-1.0, 1.0], 400_000)
    f = (rng.standard_normal(200_000) * np.exp2(rng.integers(-126, 127, 200_000))).astype(np.float32)
    fd = f.astype(np.float64)
    near = np.r_[fd, np.nextafter(fd, np.inf), np.nextafter(fd, -np.inf)]
    fmax = float(np.finfo(np.float32).max)
    edges = []
    for v in (fmax, 2.0**128, 2.0**-126, 2.0**-149, 2.0**127, 1.0, 0.61):
        for w in (v, np.nextafter(v, np.inf), np.nextafter(v, 0.0)):
            edges += [w, -w]
    edges += [0.0, -0.0, np.inf, -np.inf, np.nan, 1e300, -1e300, 1e-300, -1e-300]
    x = np.r_[pat, logu, near, np.array(edges)]
    out = prover.selftest_round_to_floats(x)
    ours, ref = out[:, :2], out[:, 2:]
    both_nan = np.isnan(ours) & np.isnan(ref)
    same = (ours.view(np.uint32) == ref.view(np.uint32)) | both_nan
    bad = np.nonzero(~same.all(axis=1))[0]
    assert len(bad) == 0, (x[bad[:5]], ours[bad[:5]], ref[bad[:5]])
