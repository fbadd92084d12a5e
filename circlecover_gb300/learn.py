"""Learned strategy ordering: records, training and evaluation on the GPU.

Records are (box, criterion, verdict) triples from the plain evaluation of
seeded tight boxes (cc_tight_eval): per box, bit k of the label is "criterion
k certifies the box" (k = 0..5, CC_TV_* order) and bit 6 is "no criterion
certifies it and R is not empty" (the box is critical: the split target).
Features, the training steps (forward, backward, Adam) and the inference run
in the library's own CUDA kernels (cc_mlp_*); torch only holds device
buffers.  `compare_orders` then runs the first-success evaluation of new
boxes in the plain order and with the network's most likely criterion first,
and checks that both decide exactly the same boxes.

For the proof itself, `proof_records` logs a sample of the r3 cells a plain
(prepared-form) run of the tight proof splits, expands each into its leaf
boxes and labels them with the plain evaluation; a network trained on them
orders the leaf criteria of `compare_proof`'s learned run
(CC_PROVE_LEARNED), which must find exactly the plain run's criticals.
"""
import time

import numpy as np

from . import workloads as W

LABEL_BITS = 7


def labels_from_masks(masks):
    """Training targets from cc_tight_eval verdict masks."""
    m = np.asarray(masks, dtype=np.uint32)
    critical = (m & 0x7F) == 0
    return ((m & 0x3F) | (critical.astype(np.uint32) << 6)).astype(np.uint32)


def record_boxes(n, seed, near_critical_share=0.5):
    """Seeded tight boxes: the criteria microbench distribution mixed with
    near-critical boxes (total weight within 1e-4 of the critical weight)."""
    k = int(n * near_critical_share)
    parts = [W.tight_microbench(n - k, seed=seed)]
    if k:
        parts.append(W.tight_near_critical(k, seed=seed + 1))
    return np.concatenate(parts)


class Records:
    """Device-resident features, labels and boxes (SoA) of one record set."""

    def __init__(self, prover, boxes):
        import torch
        self.n = len(boxes)
        self.boxes = boxes
        self.masks = prover.tight_eval(boxes)
        self.labels_np = labels_from_masks(self.masks)
        self.soa = torch.from_numpy(W.to_soa(boxes)).cuda()
        self.feat = torch.empty(self.n * 10, dtype=torch.float32, device="cuda")
        torch.cuda.synchronize()
        prover.mlp_features(self.soa.data_ptr(), self.n, self.feat.data_ptr())
        self.labels = torch.from_numpy(self.labels_np.view(np.int32)).cuda()
        torch.cuda.synchronize()


def train(prover, rec, epochs=4, batch=8192, lr=3e-3, seed=0, log=None):
    """Adam over shuffled minibatches; returns the mean loss of each epoch."""
    import torch
    gen = torch.Generator(device="cuda")
    gen.manual_seed(seed)
    feat = rec.feat.view(rec.n, 10)
    history = []
    for ep in range(epochs):
        perm = torch.randperm(rec.n, device="cuda", generator=gen)
        total, steps = 0.0, 0
        for b0 in range(0, rec.n, batch):
            idx = perm[b0:b0 + batch]
            f = feat[idx].contiguous()
            y = rec.labels[idx].contiguous()
            torch.cuda.synchronize()
            total += prover.mlp_train_step(f.data_ptr(), y.data_ptr(), len(idx), lr)
            steps += 1
        history.append(total / steps)
        if log:
            log("epoch %d: mean loss %.4f" % (ep, history[-1]))
    return history


def predict(prover, rec):
    """Logits (n x 8, column 7 unused) on the host."""
    import torch
    logits = torch.empty(rec.n * 8, dtype=torch.float32, device="cuda")
    torch.cuda.synchronize()
    prover.mlp_infer(rec.feat.data_ptr(), rec.n, logits.data_ptr())
    return logits.view(rec.n, 8).cpu().numpy()


def prediction_report(logits, labels):
    """Error rate of each output (threshold 0), and how often the most likely
    criterion really certifies the box, against how often the first
    criterion of the plain order does."""
    y = ((np.asarray(labels, dtype=np.uint32)[:, None] >> np.arange(LABEL_BITS)) & 1).astype(bool)
    pred = logits[:, :LABEL_BITS] > 0
    err = (pred != y).mean(axis=0)
    top = logits[:, :6].argmax(axis=1)
    top_ok = y[np.arange(len(y)), top]
    certified = y[:, :6].any(axis=1)
    return {"error_rate_per_output": [float(e) for e in err],
            "split_error_rate": float(err[6]),
            "top1_certifies": float(top_ok[certified].mean()) if certified.any() else 0.0,
            "plain_first_certifies": float(y[certified, 0].mean()) if certified.any() else 0.0}


def compare_orders(prover, rec, reps=3):
    """First-success evaluation in the plain order and in the learned order
    on the same boxes: wall time (device, after a warm-up), mean steps run,
    and whether both decide exactly the same boxes (decided vs critical)."""
    import torch
    out_p = torch.empty(rec.n, dtype=torch.uint8, device="cuda")
    out_l = torch.empty(rec.n, dtype=torch.uint8, device="cuda")
    ev_p = torch.empty(rec.n, dtype=torch.uint8, device="cuda")
    ev_l = torch.empty(rec.n, dtype=torch.uint8, device="cuda")
    res = {}
    for name, learned, out, ev in (("plain", False, out_p, ev_p), ("learned", True, out_l, ev_l)):
        prover.tight_first(rec.soa.data_ptr(), rec.n, out.data_ptr(), ev.data_ptr(), learned=learned)
        best = float("inf")
        for _ in range(reps):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            prover.tight_first(rec.soa.data_ptr(), rec.n, out.data_ptr(), ev.data_ptr(), learned=learned)
            torch.cuda.synchronize()
            best = min(best, time.perf_counter() - t0)
        res[name] = best
    op, ol = out_p.cpu().numpy(), out_l.cpu().numpy()
    crit_p, crit_l = (op & 0x7F) == 7, (ol & 0x7F) == 7
    trapped = int(((op & 0x80) != 0).sum() + ((ol & 0x80) != 0).sum())
    return {"boxes": rec.n, "plain_s": res["plain"], "learned_s": res["learned"],
            "speedup": res["plain"] / res["learned"],
            "plain_mean_steps": float(ev_p.float().mean().item()),
            "learned_mean_steps": float(ev_l.float().mean().item()),
            "same_decisions": bool(np.array_equal(crit_p, crit_l)), "critical": int(crit_p.sum()),
            "trapped": trapped, "outcomes_plain": op, "outcomes_learned": ol}


def leaves_of_cells(cells, s4, per_cell=None, seed=0):
    """Leaf boxes (r4 split into s4 equal pieces) of logged cells; with
    per_cell, a seeded sample of that many leaves per cell."""
    n = len(cells)
    k = s4 if per_cell is None else min(per_cell, s4)
    rng = np.random.default_rng(seed)
    idx = np.tile(np.arange(s4), (n, 1)) if per_cell is None else np.stack(
        [rng.choice(s4, k, replace=False) for _ in range(n)])
    lo = cells["r"][:, 3, 0][:, None]
    hi = cells["r"][:, 3, 1][:, None]
    step = (hi - lo) / s4
    out = np.repeat(cells, k)
    r4lo = (lo + step * idx).reshape(-1)
    r4hi = np.where(idx + 1 == s4, hi, lo + step * (idx + 1)).reshape(-1)
    out["r"][:, 3, 0] = r4lo
    out["r"][:, 3, 1] = r4hi
    return out


def proof_records(prover, root, grid, per_cell=16, max_cells=1 << 17, seed=0):
    """Records from the plain proof: its logged r3 cells expanded to leaves."""
    prover.tight_find_critical_intervals(root, grid, log_cells=True)
    cells, s4 = prover.tight_cell_log()
    if len(cells) > max_cells:
        cells = cells[np.random.default_rng(seed).choice(len(cells), max_cells, replace=False)]
    return Records(prover, leaves_of_cells(cells, s4, per_cell=per_cell, seed=seed)), len(cells)


def compare_proof(prover, root, grid, reps=1):
    """The tight proof in the prepared form with the plain leaf order and
    with the learned one: wall time (best of reps, after a warm-up run) and
    whether criticals, generation sizes and leaf counts agree."""
    prover.tight_find_critical_intervals(root, grid)
    res = {}
    for name, learned in (("batched", False), ("learned", True)):
        best, out = float("inf"), None
        for _ in range(reps):
            t0 = time.perf_counter()
            out = prover.tight_find_critical_intervals(root, grid, learned=learned)
            best = min(best, time.perf_counter() - t0)
        res[name] = (best, out)
    (tb, (cb, sb)), (tl, (cl, sl)) = res["batched"], res["learned"]
    same = (np.array_equal(cb.view(np.uint64), cl.view(np.uint64)) and sb["gen_sizes"] == sl["gen_sizes"]
            and sb["leaf_evals"] == sl["leaf_evals"] and sb["trapped_leaves"] == sl["trapped_leaves"])
    return {"batched_s": tb, "learned_s": tl, "speedup": tb / tl, "leaves": sb["leaf_evals"],
            "criticals": int(len(cb)), "same_criticals": bool(same),
            "leaf_outcomes_batched": sb["counts"][3][:7], "leaf_outcomes_learned": sl["counts"][3][:7]}
