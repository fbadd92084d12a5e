"""Sharding the proofs over processes: every generation's tasks split into
contiguous ranges over the ranks of a gloo process group, criticals
all-gathered in rank order (and, for the size-bound proof, merged again over
the whole generation).  Checked on the CPU (the oracle port computes each
rank's range) against the single-process proofs of the golden fixtures: same
criticals, same generation sizes, same summed trace.  On a GPU the same
drivers take Prover.tight_generation and Prover.sb_generation."""
import json
import os
import socket

import numpy as np
import pytest

from conftest import GOLDEN, box_from_hex, boxes_from_hex
from circlecover_gb300 import distributed as D


def test_task_ranges_partition():
    for n in (0, 1, 7, 64, 1000):
        for world in (1, 2, 3, 5):
            ranges = [D.task_range(n, r, world) for r in range(world)]
            assert ranges[0][0] == 0 and ranges[-1][1] == n
            assert all(ranges[i][1] == ranges[i + 1][0] for i in range(world - 1))
            assert max(h - l for l, h in ranges) - min(h - l for l, h in ranges) <= 1


def free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, case, out_dir):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    from oracle import oracle as O
    p = O.Port()

    def gather(obj):
        out = [None] * world
        dist.all_gather_object(out, obj)
        return out

    def generation(parents, k, splits, lo, hi):
        return p.tight_generation(parents, k, splits, lo, hi, threads=2)

    crit, st = D.prove_sharded(generation, box_from_hex(case["root"]), case["la_init"], case["r_init"], case["gens"],
                               case["r_gen"], rank, world, gather)
    np.save(os.path.join(out_dir, "crit%d.npy" % rank), crit)
    with open(os.path.join(out_dir, "stats%d.json" % rank), "w") as f:
        json.dump({k: v for k, v in st.items()}, f)
    dist.barrier()
    dist.destroy_process_group()


@pytest.mark.parametrize("world", [2, 3])
def test_sharded_proof_equals_single_process(tmp_path, world):
    import torch.multiprocessing as mp
    with open(os.path.join(GOLDEN, "tight_prove_golden.json")) as f:
        case = json.load(f)["cases"][3]  # three refinement generations
    mp.spawn(_rank_main, args=(world, free_port(), case, str(tmp_path)), nprocs=world, join=True)
    want = boxes_from_hex(case["criticals"])
    for r in range(world):
        crit = np.load(tmp_path / ("crit%d.npy" % r))
        st = json.load(open(tmp_path / ("stats%d.json" % r)))
        assert np.array_equal(crit.view(np.uint64), want.view(np.uint64))
        assert st["gen_sizes"] == case["stats"]["gen_sizes"]
        assert st["digest"] == case["stats"]["digest"]
        assert st["counts"] == case["stats"]["counts"]
        assert st["leaf_evals"] == case["stats"]["leaf_evals"]


def _sb_rank_main(rank, world, port, case, out_dir):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    from oracle import oracle as O
    from test_sb_prove import box6_from_hex
    p = O.Port()

    def gather(obj):
        out = [None] * world
        dist.all_gather_object(out, obj)
        return out

    def generation(parents, gen, k, splits, lo, hi):
        return p.sb_generation(parents, gen, k, splits, lo, hi, threads=2)

    crit, flags, st = D.prove_sb_sharded(generation, box6_from_hex(case["root"]), case["la_init"], case["r_init"],
                                         case["la_gen"], case["r_gen"], case["gens"], rank, world, gather)
    np.save(os.path.join(out_dir, "crit%d.npy" % rank), crit)
    np.save(os.path.join(out_dir, "flags%d.npy" % rank), flags)
    with open(os.path.join(out_dir, "stats%d.json" % rank), "w") as f:
        json.dump({k: v for k, v in st.items()}, f)
    dist.barrier()
    dist.destroy_process_group()


@pytest.mark.parametrize("name,world", [("three_generations", 2), ("three_generations", 3), ("mixed_disks", 2)])
def test_sharded_size_bound_proof_equals_single_process(tmp_path, name, world):
    """The size-bound proof sharded over gloo ranks, generation by generation
    (the three-generation case uses all three merge widths), equals the
    reference's single-process proof in the golden fixture."""
    import torch.multiprocessing as mp
    from test_sb_prove import boxes6_from_hex
    with open(os.path.join(GOLDEN, "sb_prove_golden.json")) as f:
        case = next(c for c in json.load(f)["cases"] if c["name"] == name)
    mp.spawn(_sb_rank_main, args=(world, free_port(), case, str(tmp_path)), nprocs=world, join=True)
    want = boxes6_from_hex(case["criticals"])
    for r in range(world):
        crit = np.load(tmp_path / ("crit%d.npy" % r))
        flags = np.load(tmp_path / ("flags%d.npy" % r))
        st = json.load(open(tmp_path / ("stats%d.json" % r)))
        assert len(crit) == len(want) and np.array_equal(crit.view(np.uint64), want.view(np.uint64))
        assert [int(x) for x in flags] == case["flags"]
        assert st["gen_sizes"] == case["stats"]["gen_sizes"]
        assert st["digest"] == case["stats"]["digest"]
        assert st["leaf_evals"] == case["stats"]["leaf_evals"]
        for k in ("task_counts", "cell_counts", "leaf_counts", "trapped_leaves"):
            assert st[k] == case["stats"][k], k


@pytest.mark.gpu
def test_gpu_generation_ranges_concatenate(prover, golden_prove):
    """On one GPU: the generation entry point over two task ranges gives the
    whole generation's criticals and trace when concatenated and summed."""
    import circlecover_gb300 as cg
    c = golden_prove[3]
    g = cg.make_grid(c["la_init"], c["r_init"], c["gens"], c["r_gen"])

    full, st_full = prover.tight_find_critical_intervals(box_from_hex(c["root"]), g)
    crit, st = D.prove_sharded(lambda *a: _two_ranges(prover, *a), box_from_hex(c["root"]), c["la_init"], c["r_init"],
                               c["gens"], c["r_gen"], 0, 1, lambda obj: [obj])
    assert np.array_equal(crit.view(np.uint64), full.view(np.uint64))
    assert st["digest"] == st_full["digest"] and st["gen_sizes"] == st_full["gen_sizes"]


def _two_ranges(prover, parents, k, splits, lo, hi):
    """A generation computed as two half ranges, concatenated in order."""
    mid = (lo + min(hi, len(parents) * k)) // 2
    a, sa = prover.tight_generation(parents, k, splits, lo, mid)
    b, sb = prover.tight_generation(parents, k, splits, mid, hi)
    st = dict(sa)
    st["counts"] = (np.array(sa["counts"], dtype=np.uint64) + np.array(sb["counts"], dtype=np.uint64)).tolist()
    st["digest"] = (sa["digest"] + sb["digest"]) % (1 << 64)
    st["leaf_evals"] = sa["leaf_evals"] + sb["leaf_evals"]
    st["trapped_leaves"] = sa["trapped_leaves"] + sb["trapped_leaves"]
    return np.concatenate([a, b]), st


@pytest.mark.gpu
def test_gpu_sharded_size_bound_proof(prover):
    """On one GPU: the size-bound driver with three ranks emulated in one
    process (each rank's range by cc_sb_generation, gathered in rank order)
    gives the reference's proof of the three-generation golden case."""
    from test_sb_prove import box6_from_hex, boxes6_from_hex
    with open(os.path.join(GOLDEN, "sb_prove_golden.json")) as f:
        case = next(c for c in json.load(f)["cases"] if c["name"] == "three_generations")
    world = 3

    def gen_all_ranks(parents, gen, k, splits, lo, hi):  # lo, hi of rank 0; the others computed here
        n = len(parents) * k * splits[0] * splits[1]
        return [prover.sb_generation(parents, gen, k, splits, *D.task_range(n, r, world)) for r in range(world)]

    state = {}

    def generation(parents, gen, k, splits, lo, hi):
        state["parts"] = gen_all_ranks(parents, gen, k, splits, lo, hi)
        return state["parts"][0]

    def gather(obj):
        return [obj] + [(p[0], p[1], p[2]) for p in state["parts"][1:]]

    crit, flags, st = D.prove_sb_sharded(generation, box6_from_hex(case["root"]), case["la_init"], case["r_init"],
                                         case["la_gen"], case["r_gen"], case["gens"], 0, world, gather)
    want = boxes6_from_hex(case["criticals"])
    assert len(crit) == len(want) and np.array_equal(crit.view(np.uint64), want.view(np.uint64))
    assert [int(x) for x in flags] == case["flags"]
    assert st["gen_sizes"] == case["stats"]["gen_sizes"] and st["digest"] == case["stats"]["digest"]
