"""Sharding a tight proof over processes (one GPU per process).

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
"""
import numpy as np

from .workloads import TIGHT_BOX


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
