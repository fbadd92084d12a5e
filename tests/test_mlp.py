"""Learned strategy ordering: the float64 oracle of the network checked by
finite differences (CPU), the GPU training kernels' gradients against it, the
tensor-core inference against a BF16 emulation, training progress, and the
first-success evaluation in both orders (same decisions, consistent with the
plain verdict masks)."""
import numpy as np
import pytest

from oracle import mlp_ref as M


def random_case(n, seed):
    rng = np.random.default_rng(seed)
    w = (rng.standard_normal(M.P) * 0.2).astype(np.float32)
    x = rng.standard_normal((n, M.F)).astype(np.float32)
    labels = rng.integers(0, 1 << M.O, n).astype(np.uint32)
    return w, x, labels


def test_oracle_gradient_matches_finite_differences():
    w, x, labels = random_case(40, 1)
    w = w.astype(np.float64)
    g = M.gradient(w, x, labels)
    rng = np.random.default_rng(2)
    for p in rng.choice(M.P, 60, replace=False):
        e = np.zeros(M.P)
        e[p] = 1e-6
        fd = (M.loss(w + e, x, labels) - M.loss(w - e, x, labels)) / 2e-6
        assert abs(fd - g[p]) <= 1e-6 + 1e-4 * abs(fd)


def test_bf16_rounding_is_nearest_even():
    v = np.array([1.0, 1.00390625, 1.005859375, 1.0078125, -3.14159], dtype=np.float32)
    r = M.bf16(v)
    assert r[0] == 1.0 and r[1] == 1.0 and r[2] == np.float32(1.0078125) and r[3] == np.float32(1.0078125)
    assert abs(r[4] + 3.140625) < 1e-6


@pytest.mark.gpu
def test_gpu_gradients_match_oracle(prover):
    import torch
    w, x, labels = random_case(300, 3)  # not a multiple of the 128-sample block
    prover.mlp_init(0)
    prover.mlp_set_weights(w)
    xf = torch.from_numpy(x.reshape(-1)).cuda()
    yl = torch.from_numpy(labels.view(np.int32)).cuda()
    torch.cuda.synchronize()
    g, loss = prover.mlp_gradients(xf.data_ptr(), yl.data_ptr(), len(x))
    want = M.gradient(w.astype(np.float64), x, labels)
    assert abs(loss - M.loss(w.astype(np.float64), x, labels)) < 1e-4 * max(1.0, abs(loss))
    scale = np.abs(want).max()
    assert np.abs(g - want).max() <= 1e-4 * scale + 1e-7


@pytest.mark.gpu
def test_gpu_tensor_core_inference_matches_bf16_emulation(prover):
    import torch
    w, x, labels = random_case(1000, 4)
    prover.mlp_init(0)
    prover.mlp_set_weights(w)
    xf = torch.from_numpy(x.reshape(-1)).cuda()
    out = torch.zeros(len(x) * 8, dtype=torch.float32, device="cuda")
    torch.cuda.synchronize()
    prover.mlp_infer(xf.data_ptr(), len(x), out.data_ptr())
    got = out.view(len(x), 8).cpu().numpy()[:, :M.O]
    want = M.infer_bf16(w, x)
    exact = M.forward(w.astype(np.float64), x)[0]
    tol = 2e-3 * np.abs(want).max() + 1e-3
    assert np.abs(got - want).max() <= tol  # summation order only
    assert np.abs(got - exact).max() <= 0.1 * np.abs(exact).max()  # BF16 vs float64


@pytest.mark.gpu
def test_gpu_training_learns_the_verdicts_and_orders_identically(prover):
    from circlecover_gb300 import learn
    prover.mlp_init(7)
    train_rec = learn.Records(prover, learn.record_boxes(1 << 16, seed=101))
    hist = learn.train(prover, train_rec, epochs=6, batch=4096, lr=3e-3)
    assert hist[-1] < 0.7 * hist[0]
    test_rec = learn.Records(prover, learn.record_boxes(1 << 15, seed=202))
    rep = learn.prediction_report(learn.predict(prover, test_rec), test_rec.labels_np)
    base = test_rec.labels_np[:, None] >> np.arange(7) & 1
    prior_err = np.minimum(base.mean(0), 1 - base.mean(0))
    # every output beats always answering its majority class
    assert all(e <= p + 1e-9 for e, p in zip(rep["error_rate_per_output"], prior_err))
    cmp = learn.compare_orders(prover, test_rec, reps=1)
    assert cmp["same_decisions"]
    # the plain first-success outcome is the first set verdict bit in the nesting order
    m = test_rec.masks
    order = [0, 1, 2, 6, 3, 4, 5]
    first = np.full(len(m), 7)
    for k in reversed(order):
        first = np.where((m >> k) & 1 == 1, k, first)
    assert np.array_equal(cmp["outcomes_plain"] & 0x7F, first)


@pytest.mark.gpu
def test_gpu_learned_proof_finds_the_same_criticals(prover, golden_prove):
    """The tight proof with the learned leaf order (CC_PROVE_LEARNED), its
    network trained on records from the plain proof's own cells, finds the
    reference's criticals, generation sizes and leaf count on every golden
    case."""
    import circlecover_gb300 as cg
    from circlecover_gb300 import learn
    from circlecover_gb300 import workloads as W
    from conftest import box_from_hex, boxes_from_hex
    prover.mlp_init(5)
    rec, ncells = learn.proof_records(prover, W.tight_root(1.0, 1.1), cg.make_grid(16, (16, 32, 32, 32)), per_cell=8)
    assert ncells > 0
    learn.train(prover, rec, epochs=3, batch=4096)
    reordered = 0
    for c in golden_prove:
        g = cg.make_grid(c["la_init"], c["r_init"], c["gens"], c["r_gen"])
        crit, st = prover.tight_find_critical_intervals(box_from_hex(c["root"]), g, learned=True)
        want = boxes_from_hex(c["criticals"])
        assert np.array_equal(crit.view(np.uint64), want.view(np.uint64))
        assert st["gen_sizes"] == c["stats"]["gen_sizes"] and st["leaf_evals"] == c["stats"]["leaf_evals"]
        reordered += st["counts"][3][3] - c["stats"]["counts"][3][3]
    assert reordered > 0  # the leaf criterion certified leaves the 2x2 criterion used to


@pytest.mark.gpu
def test_gpu_learned_order_saves_leaf_work(prover):
    """What the network gains: on the initial pass of the small plain-method
    workload (lambda in [1, 1.1], 64 lambda pieces, r splits 32 x 64^3) the
    learned leaf order puts the prepared leaf criterion before the 2x2 one in
    the cells where it certifies, so the FP32-first 2x2 evaluations the
    batched form makes (nearly all of them "false") mostly disappear; the
    criticals and the leaf count are the same.  (Wall times, about 20 ms each
    here, are printed; the assertion on them only excludes a large loss.)"""
    import time
    import circlecover_gb300 as cg
    from circlecover_gb300 import learn
    from circlecover_gb300 import workloads as W
    root = W.tight_root(1.0, 1.1)
    grid = cg.make_grid(64, (32, 64, 64, 64))
    prover.mlp_init(13)
    rec, ncells = learn.proof_records(prover, root, grid, per_cell=8)
    learn.train(prover, rec, epochs=3, batch=4096)
    res = {}
    for name, kw in (("batched", {}), ("learned", {"learned": True})):
        prover.tight_find_critical_intervals(root, grid, **kw)  # warm
        best = float("inf")
        for _ in range(2):
            t0 = time.perf_counter()
            crit, st = prover.tight_find_critical_intervals(root, grid, **kw)
            best = min(best, time.perf_counter() - t0)
        res[name] = (best, crit, st)
    (tb, cb, sb), (tl, cl, sl) = res["batched"], res["learned"]
    assert np.array_equal(cb.view(np.uint64), cl.view(np.uint64)) and sb["leaf_evals"] == sl["leaf_evals"]
    fp32_b, fp32_l = sum(sb["fp32_first"][:3]), sum(sl["fp32_first"][:3])
    print("FP32-first leaf evaluations: batched %d, learned %d; seconds: batched %.3f, learned %.3f"
          % (fp32_b, fp32_l, tb, tl))
    assert fp32_l < 0.2 * fp32_b
    assert tl < 1.5 * tb
