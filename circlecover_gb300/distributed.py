"""Sharding the proofs over processes (one GPU per process).

Every task of a generation (one lambda piece of one parent box) is
independent, so a generation splits into contiguous task ranges, one per
rank, with no exchange inside it.  After each generation the ranks
all-gather their criticals in rank order; because each range's criticals
come out in task order and merged per task (as the reference merges them),
the concatenation is exactly the whole generation's output and becomes every
rank's list of parents for the next generation.  The per-rank trace counts
and digests add up to the single-process trace.  This is the only
collective the proof needs (one all-gather per generation); there is no
device-side communication.

`prove_sharded` takes the generation function as an argument: on a GPU it
is `Prover.tight_generation`; the tests plug in the CPU oracle to check the
logic with gloo process groups.

The size-bound proof shards the same way over its (parent, lambda piece, r1
piece, r2 piece) tasks (`prove_sb_sharded`, with `Prover.sb_generation` on
a GPU).  Its generations end with a merge over all the generation's
criticals (sort, then join the boxes with equal lambda and equal leading
radii), which each rank applies to its own range; merging the rank-ordered
concatenation of those merged lists again gives the merge of the whole
generation (the join is a hull over the boxes of one key, and a key's boxes
are consecutive after the sort), so the gathered result is the
single-process one.
"""
import numpy as np

from .workloads import SB_BOX, TIGHT_BOX


def task_range(n_tasks, rank, world):
    """Contiguous block [lo, hi) of n_tasks for rank (sizes differ by <= 1)."""
    base, extra = divmod(n_tasks, world)
    lo = rank * base + min(rank, extra)
    return lo, lo + base + (1 if rank < extra else 0)


def _add_stats(total, st):
    if total is None:
        return {k: (np.array(v, dtype=np.uint64) if k == "counts" else v)
                for k, v in st.items() if k in ("counts", "digest", "leaf_evals", "trapped_leaves")}
    total["counts"] = total["counts"] + np.array(st["counts"], dtype=np.uint64)
    total["digest"] = (total["digest"] + st["digest"]) % (1 << 64)
    total["leaf_evals"] += st["leaf_evals"]
    total["trapped_leaves"] += st["trapped_leaves"]
    return total


def prove_sharded(generation, root, la_init, r_init, gens, r_gen, rank, world, all_gather):
    """The tight proof (root, split counts as cc_tight_grid) with every
    generation's tasks sharded over `world` ranks.

    generation(parents, la_splits, r_splits, lo, hi) -> (criticals, stats)
    all_gather(obj) -> list of every rank's obj, in rank order
    Returns (criticals, stats with the summed trace and gen_sizes), the same
    on every rank."""
    parents = np.asarray([root], dtype=TIGHT_BOX).reshape(-1)
    total, sizes = None, []
    schedule = [(la_init, r_init)] + [(k, r_gen) for k in gens]
    for g, (k, splits) in enumerate(schedule):
        if g > 0 and len(parents) == 0:
            break
        lo, hi = task_range(len(parents) * k, rank, world)
        crit, st = generation(parents, k, splits, lo, hi)
        parts = all_gather((np.asarray(crit, dtype=TIGHT_BOX), st))
        parents = np.concatenate([p[0] for p in parts]) if parts else np.zeros(0, dtype=TIGHT_BOX)
        for _, s in parts:
            total = _add_stats(total, s)
        sizes.append(len(parents))
    total["counts"] = total["counts"].tolist()
    total["gen_sizes"] = sizes
    total["generations_run"] = len(sizes) - 1
    return parents, total


def sb_merge_width(gen):
    """Radii kept as the merge key after generation gen
    (rectangle_size_bound.cu:351-362): 0 for the initial pass, then 2, 1, 3
    in turn."""
    return 0 if gen == 0 else (3 if gen % 3 == 0 else (2 if gen % 3 == 1 else 1))


def sb_merge(boxes, flags, n_merged):
    """merge_critical_intervals<N> (rectangle_size_bound.cu:103-130) on the
    host: sort by lambda, then radii 1..6 (each interval by lower, then upper
    bound), and join radii N+1..6 of consecutive boxes with equal lambda and
    equal radii 1..N (the hull; trap flags OR-ed)."""
    boxes = np.asarray(boxes, dtype=SB_BOX).reshape(-1)
    flags = np.asarray(flags, dtype=np.uint32).reshape(-1)
    if not len(boxes):
        return boxes.copy(), flags.copy()
    keys = [boxes["la"][:, 0], boxes["la"][:, 1]]
    for i in range(6):
        keys += [boxes["r"][:, i, 0], boxes["r"][:, i, 1]]
    order = np.lexsort(tuple(reversed(keys)))
    la, r = boxes["la"], boxes["r"]
    out = np.zeros(len(boxes), dtype=SB_BOX)
    out_flags = np.zeros(len(boxes), dtype=np.uint32)
    m = 0  # boxes in out
    for j in order:
        if m:
            p = m - 1
            same = out["la"][p, 0] == la[j, 0] and out["la"][p, 1] == la[j, 1]
            for i in range(n_merged):
                same = same and out["r"][p, i, 0] == r[j, i, 0] and out["r"][p, i, 1] == r[j, i, 1]
            if same:
                for i in range(n_merged, 6):
                    if r[j, i, 0] < out["r"][p, i, 0]:
                        out["r"][p, i, 0] = r[j, i, 0]
                    if r[j, i, 1] > out["r"][p, i, 1]:
                        out["r"][p, i, 1] = r[j, i, 1]
                out_flags[p] |= flags[j]
                continue
        out[m] = boxes[j]
        out_flags[m] = flags[j]
        m += 1
    return out[:m], out_flags[:m]


def _add_sb_stats(total, st):
    keys = ("task_counts", "cell_counts", "leaf_counts")
    if total is None:
        total = {k: np.zeros(len(st[k]), dtype=np.uint64) for k in keys}
        total.update(digest=0, leaf_evals=0, trapped_leaves=0)
    for k in keys:
        total[k] = total[k] + np.array(st[k], dtype=np.uint64)
    total["digest"] = (total["digest"] + st["digest"]) % (1 << 64)
    total["leaf_evals"] += st["leaf_evals"]
    total["trapped_leaves"] += st["trapped_leaves"]
    return total


def prove_sb_sharded(generation, root, la_init, r_init, la_gen, r_gen, gens, rank, world, all_gather):
    """The size-bound proof (root, split counts as cc_sb_grid) with every
    generation's tasks sharded over `world` ranks.

    generation(parents, gen, la_splits, r_splits, lo, hi) -> (criticals, flags, stats)
    all_gather(obj) -> list of every rank's obj, in rank order
    Returns (criticals, flags, stats with the summed trace and gen_sizes), the
    same on every rank."""
    parents = np.asarray([root], dtype=SB_BOX).reshape(-1)
    pflags = np.zeros(0, dtype=np.uint32)
    total, sizes = None, []
    for g in range(gens + 1):
        if g > 0 and len(parents) == 0:
            break
        k, rs = (la_init, r_init) if g == 0 else (la_gen, r_gen)
        lo, hi = task_range(len(parents) * k * rs[0] * rs[1], rank, world)
        crit, flags, st = generation(parents, g, k, rs, lo, hi)
        parts = all_gather((np.asarray(crit, dtype=SB_BOX), np.asarray(flags, dtype=np.uint32), st))
        parents, pflags = sb_merge(np.concatenate([p[0] for p in parts]), np.concatenate([p[1] for p in parts]),
                                   sb_merge_width(g))
        for _, _, s in parts:
            total = _add_sb_stats(total, s)
        sizes.append(len(parents))
    for k in ("task_counts", "cell_counts", "leaf_counts"):
        total[k] = total[k].tolist()
    total["gen_sizes"] = sizes
    total["generations_run"] = len(sizes) - 1
    return parents, pflags, total
