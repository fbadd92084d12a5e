"""GPU tier: adaptive refinement of near-critical tight boxes
(cc_tight_refine) against the same refinement driven by the CPU oracle's
verdict masks: per level, the boxes no criterion certifies and that are not
empty are bisected along lambda, r1, r2, r3, r4 in turn (mid = 0.5 lo + 0.5
hi, rounded to nearest), the first max_live / 2 of them in level order, the
halves listed in the order of their boxes; trapped boxes, the undecided
boxes of the last level and the boxes past the cap are the criticals.  The
GPU's criticals (in order), flags and per-level counts equal the
oracle-driven ones."""
import numpy as np
import pytest

from circlecover_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def oracle_refine(port, boxes, max_depth, max_live=1 << 26):
    crit, flags, live, decided = [], [], [], []
    cur = boxes.copy()
    for d in range(max_depth + 1):
        if not len(cur):
            break
        m = port.tight_eval(cur, threads=16)
        trapped = (m >> 31) != 0
        done = ~trapped & ((m & 0x7F) != 0)
        live.append(len(cur))
        decided.append(int(done.sum()))
        last = d == max_depth
        cand = ~trapped & ~done & (not last)
        cut = cand & (np.cumsum(cand) > max_live // 2)
        keep = trapped | (~done & last) | cut
        crit.append(cur[keep])
        flags.append(np.where(trapped[keep], 1, np.where(cut[keep], 3, 2)).astype(np.uint32))
        split = cur[cand & ~cut]
        dim = d % 5
        lo_half, hi_half = split.copy(), split.copy()
        if dim == 0:
            v = split["la"]
            mid = 0.5 * v[:, 0] + 0.5 * v[:, 1]
            lo_half["la"][:, 1] = mid
            hi_half["la"][:, 0] = mid
        else:
            v = split["r"][:, dim - 1]
            mid = 0.5 * v[:, 0] + 0.5 * v[:, 1]
            lo_half["r"][:, dim - 1, 1] = mid
            hi_half["r"][:, dim - 1, 0] = mid
        nxt = np.empty(2 * len(split), dtype=W.TIGHT_BOX)
        nxt[0::2], nxt[1::2] = lo_half, hi_half
        cur = nxt
    return np.concatenate(crit), np.concatenate(flags), live, decided


def same_bits(a, b):
    return len(a) == len(b) and np.array_equal(a.view(np.uint64), b.view(np.uint64))


def test_refine_equals_oracle_driven_refinement(prover, port):
    boxes = W.tight_near_critical(2000, seed=505)
    got, gflags, st = prover.tight_refine(boxes, max_depth=7)
    want, wflags, live, decided = oracle_refine(port, boxes, 7)
    assert st["live"] == live and st["decided"] == decided
    assert same_bits(got, want) and np.array_equal(gflags, wflags)
    assert st["depths_run"] == len(live) and not st["stopped_at_cap"]


def test_refine_population_cap_cuts_in_level_order(prover, port):
    """A cap of 6,000 live boxes: the refinement still runs to its depth, the
    boxes past the cap are kept (flag 3) exactly as the sequential model
    keeps them, and a second run gives the same output."""
    boxes = W.tight_near_critical(4000, seed=506)
    got, flags, st = prover.tight_refine(boxes, max_depth=12, max_live=6000)
    assert st["stopped_at_cap"] and max(st["live"]) <= 6000 and sum(st["cut"]) == int((flags == 3).sum()) > 0
    want, wflags, live, decided = oracle_refine(port, boxes, 12, max_live=6000)
    assert st["live"] == live and st["decided"] == decided
    assert same_bits(got, want) and np.array_equal(flags, wflags)
    again, aflags, _ = prover.tight_refine(boxes, max_depth=12, max_live=6000)
    assert same_bits(again, got) and np.array_equal(aflags, flags)


def test_refine_orders_decide_the_same_boxes(prover):
    """First-success refinement (plain order, and the network's choice first)
    decides exactly the boxes the certified masks decide at every level, so
    live and decided counts and the criticals agree; it reports its steps."""
    from circlecover_gb300 import learn
    boxes = W.tight_near_critical(3000, seed=507)
    got, gflags, st = prover.tight_refine(boxes, max_depth=9)
    assert st["order"] == 0 and sum(st["fp64_boxes"]) + sum(st["cover_jobs"]) > 0
    assert all(f <= l for f, l in zip(st["fp64_boxes"], st["live"]))
    prover.mlp_init(9)
    learn.train(prover, learn.Records(prover, W.tight_near_critical(1 << 14, seed=508)), epochs=1, batch=4096)
    for order in ("first_plain", "first_learned"):
        c, f, s = prover.tight_refine(boxes, max_depth=9, order=order)
        assert s["order"] == (1 if order == "first_plain" else 2)
        assert all(k >= l - d for k, l, d in zip(s["steps"], s["live"], s["decided"])), order
        assert all(k <= 32 * w and w <= k for k, w in zip(s["steps"], s["warp_max_steps"])), order
        # a trap site reached after the certifying criterion keeps a box in
        # the masks order only; without traps both refinements are the same
        if not (gflags == 1).any() and not (f == 1).any():
            assert s["live"] == st["live"] and s["decided"] == st["decided"], order
            assert same_bits(c, got) and np.array_equal(f, gflags), order
        else:
            assert s["decided"][0] >= st["decided"][0], order
    prover.tight_refine(boxes[:1], max_depth=0)  # back to the default order
