"""Benchmark of the tight-rectangle criteria hot path on GB300.

Workload (one "step"): the batched-criteria microbench -- 2**24 seeded
synthetic boxes (lambda ~ U[1,4], radii and widths as in
circlecover_gb300.workloads.tight_microbench), all six exported tight
criteria evaluated per box, FP64 directed rounding, one verdict mask per box.
Inputs (1.34 GB SoA) are larger than L2 (129 MB), so no flush is needed
between steps.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

One JSON line on rank 0.  `value` = boxes/s with the inputs resident in HBM
(device entry point cc_tight_eval_device, CUDA events on the launching
stream); `e2e` = the same through the host entry point cc_tight_eval with host
buffers (host->device copy of the boxes and device->host copy of the masks in
the timed region).  --impl reference times the CPU implementation of the
criteria on the host cores (the reference's own code where it was built here,
otherwise the oracle's port of it) on the same workload.
"""
import argparse
import json
import os
import shutil
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

# the headline metric as named for this project; the workload it is measured
# on here is the batched criteria microbench (config.workload)
METRIC = "proof wall-time & boxes/s: learned+batched vs plain GB300, identical verdicts"
UNIT = "boxes/s"


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


class ClockSampler:
    """nvidia-smi clocks/throttle reasons sampled during the timed region."""
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.proc = None
        self.path = None

    def start(self):
        if not shutil.which("nvidia-smi"):
            return
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), "--query-gpu=" + self.FIELDS,
                                      "--format=csv,noheader,nounits", "-lms", "100"],
                                     stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)

    def stop(self):
        if not self.proc:
            return None
        time.sleep(0.15)
        self.proc.terminate()
        self.proc.wait()
        rows = [l.split(", ") for l in open(self.path).read().strip().splitlines() if l.strip()]
        os.unlink(self.path)
        sm = [float(r[1]) for r in rows if len(r) >= 9 and r[1].replace(".", "").isdigit()]
        if not sm:
            return None
        mx = max(float(r[2]) for r in rows if len(r) >= 9)
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for r in rows if len(r) >= 9 for k in range(4) if r[5 + k].strip() == "Active"})
        under_load = [s for s in sm if s > 0.3 * mx] or sm
        return {"sm_mhz": float(np.median(under_load)), "sm_max_mhz": mx, "reasons": reasons, "samples": len(sm)}


def algorithmic_ops_per_box():
    """Mean number of FP64 directed-rounding operations the REFERENCE's code
    executes per box of this workload (shim counters on the reference built
    for the host; first 2**16 boxes of the 2**24-box set), split by the kernel
    that executes them: the strip-width and gap-width bisection loops (counted
    on the port, whose loops execute the reference's operations one for one)
    and the main pass (the rest of the reference's count)."""
    z = np.load(os.path.join(ROOT, "tests", "golden", "tight_bench_ops.npz"))
    total = float(z["ops"].astype(np.float64).mean())
    cover = float(z["cover_ops"].astype(np.float64).mean())
    gaps = float(z["gaps_ops"].astype(np.float64).mean())
    # the main criteria's operations are decided by the FP32 pass, or by the
    # FP64 pass for the boxes the FP32 pass leaves to it: counted at the FP32 pass
    return total, {"k_eval_f32": total - cover - gaps, "k_eval_main": 0.0, "k_eval_cover": cover,
                   "k_eval_gaps": gaps}, z["masks"]


def ncu_traffic(kernel):
    """DRAM bytes (read + write) per full-size launch of `kernel` from the
    committed ncu summary (a line `traffic_bytes_per_launch[<kernel>]: B`)."""
    p = os.path.join(ROOT, "profiles", "tight_eval_microbench_2e24.md")
    if not os.path.exists(p):
        return None
    key = "traffic_bytes_per_launch[%s]:" % kernel
    for line in open(p):
        if line.startswith(key):
            try:
                return float(line.split(":", 1)[1])
            except ValueError:
                return None
    return None


_CPU_BOXES = {}


def cpu_baseline(n_sample, seed=1):
    """The CPU implementation on all host cores over a bounded sample of the
    workload (about 10 s of CPU work at the default sample): the reference's
    own criteria code if it was built on this host, else the oracle's port
    of it."""
    from circlecover_gb300 import workloads as W
    from oracle import oracle as O
    O.ensure_built()
    cores = os.cpu_count() or 1
    if O.ref_available():
        impl, kind = O.Ref(), "reference"
    else:
        impl, kind = O.Port(), "port"
    if (n_sample, seed) not in _CPU_BOXES:
        _CPU_BOXES[(n_sample, seed)] = W.tight_microbench(n_sample, seed=seed)
    boxes = _CPU_BOXES[(n_sample, seed)]
    impl.tight_eval(boxes[:4096], threads=cores)
    t0 = time.perf_counter()
    impl.tight_eval(boxes, threads=cores)
    dt = time.perf_counter() - t0
    return {"value": n_sample / dt, "unit": UNIT, "cores": cores, "kind": kind,
            "sample": "first %d boxes of the 2^24-box microbench (seed 1), %d threads, %.2f s" % (n_sample, cores, dt)}


def run_reference(args, ws, rank):
    if rank != 0:
        return
    steps = []
    n_sample = args.cpu_sample
    for i in range(args.warmup + args.steps):
        cb = cpu_baseline(n_sample)
        if i >= args.warmup:
            steps.append(cb)
    vals = [s["value"] for s in steps]
    v = float(np.median(vals))
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1000.0 * n_sample / v, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded, platform-independent generator)",
            "config": {"workload": "tight criteria microbench, 2^24 boxes; each CPU step a bounded sample",
                       "boxes_per_step": n_sample},
            "cpu_baseline": steps[-1] | {"value": v},
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def run_ours(args, ws, rank, local):
    import torch
    import circlecover_gb300 as cg
    from circlecover_gb300 import workloads as W

    torch.cuda.set_device(local)
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    n = 1 << args.log2n
    # weak scaling: every rank evaluates its own 2**log2n boxes
    boxes = W.tight_microbench(n, seed=1, start=rank * n)
    soa = torch.from_numpy(W.to_soa(boxes)).to("cuda")
    masks = torch.empty(n, dtype=torch.int32, device="cuda")
    prover = cg.Prover(local)
    # a dedicated (non-default) stream: the kernels launch on it and the CUDA
    # events are recorded on it
    stream = torch.cuda.Stream()
    assert stream.cuda_stream != 0

    def step():
        prover.tight_eval_device(soa.data_ptr(), n, masks.data_ptr(), stream.cuda_stream)

    def barrier():
        torch.cuda.synchronize()
        if ws > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()

    barrier()  # inputs were copied on the default stream
    tune = None
    if not args.no_autotune:  # register budget and grid of each pass, on a 2^22-box sample
        # (large enough that the bisection passes' queues, 14 % and 31 % of
        # the boxes, give every thread several jobs, as at full size)
        m = min(n, 1 << 22)
        sample = torch.from_numpy(W.to_soa(boxes[:m])).to("cuda")
        smask = torch.empty(m, dtype=torch.int32, device="cuda")
        torch.cuda.synchronize()
        tune = prover.autotune_eval(sample.data_ptr(), m, smask.data_ptr())
        del sample, smask
    for _ in range(args.warmup):
        step()
    barrier()
    launches_per_step = prover.last_launch_count
    # per-kernel CUDA events (recorded by the library on the same stream)
    prover.set_stage_timing(True)
    stage_ms = np.zeros(len(cg.EVAL_PASSES))
    clocks = ClockSampler(local)
    clocks.start()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(args.steps):
        step()
        stage_ms += np.array(prover.stage_times())
    e1.record(stream)
    barrier()
    ck = clocks.stop()
    prover.set_stage_timing(False)
    ms = e0.elapsed_time(e1) / args.steps
    stage_ms /= args.steps
    if ws > 1:
        t = torch.tensor([ms], device="cuda", dtype=torch.float64)
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        ms = float(t.item())
    value = ws * n / (ms * 1e-3)

    # correctness of the timed output: the sampled boxes' masks equal the
    # reference's (golden) masks
    ops_per_box, stage_ops, ref_masks = algorithmic_ops_per_box()
    got = masks[: len(ref_masks)].cpu().numpy().view(np.uint32)
    verified = bool(rank != 0 or np.array_equal(got, ref_masks))

    # end to end through the host entry point (host buffers, copies inside)
    e2e = None
    if not args.no_e2e:
        # inputs and results in page-locked host memory
        pinned_in = torch.empty(n * W.TIGHT_BOX.itemsize, dtype=torch.uint8, pin_memory=True)
        host_boxes = pinned_in.numpy().view(W.TIGHT_BOX)
        host_boxes[:] = boxes
        out = torch.empty(n, dtype=torch.int32, pin_memory=True).numpy().view(np.uint32)
        prover.tight_eval(host_boxes, out=out)  # warm-up at full size: the entry point's buffers grow once
        barrier()
        t0 = time.perf_counter()
        for _ in range(args.steps):
            prover.tight_eval(host_boxes, out=out)
        dt = (time.perf_counter() - t0) / args.steps
        if ws > 1:
            t = torch.tensor([dt], device="cuda", dtype=torch.float64)
            torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
            dt = float(t.item())
        verified = verified and bool(rank != 0 or np.array_equal(out[: len(ref_masks)], ref_masks))
        e2e = {"value": ws * n / dt, "unit": UNIT, "h2d_bytes_per_step": int(n * 80), "d2h_bytes_per_step": int(n * 4)}

    if rank != 0:
        prover.close()
        return
    peak = ctypes_peak(prover)
    names = list(cg.EVAL_PASSES)
    stages = {k: {"ms": float(stage_ms[i]), "ops_per_box": stage_ops[k],
                  "achieved": stage_ops[k] * n / (stage_ms[i] * 1e-3) / 1e12,
                  "frac": stage_ops[k] * n / (stage_ms[i] * 1e-3) / peak} for i, k in enumerate(names)}
    dom = names[int(np.argmax(stage_ms))]
    achieved = stage_ops[dom] * n / (stage_ms[names.index(dom)] * 1e-3)
    step_achieved = ops_per_box * n / (ms * 1e-3)
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": ms, "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded, platform-independent generator)",
        "config": {"workload": "tight criteria microbench: 2^24 boxes per GPU, lambda~U[1,4], log-uniform widths "
                               "2^-20..2^-4, total weight critical*(1+eps), eps log-uniform 1e-6..1e-1",
                   "boxes_per_gpu": n, "l2_flush": "not needed: inputs (%.2f GB) exceed L2" % (n * 80 / 1e9),
                   "layout": "SoA, 10 x n float64", "autotune": tune},
        "verified_vs_reference_masks": verified,
        "roofline": {"bound": "fp64", "kernel": dom, "achieved": achieved / 1e12, "peak": peak / 1e12,
                     "unit": "Top/s (FP64 ops)", "frac": achieved / peak, "traffic": ncu_traffic(dom),
                     "ops_per_box": stage_ops[dom], "stages": stages,
                     "step": {"achieved": step_achieved / 1e12, "frac": step_achieved / peak,
                              "ops_per_box": ops_per_box},
                     "note": "achieved = the reference's FP64 directed-rounding ops per box that this pass "
                             "settles (shim-counted on the reference) x boxes / the pass's mean CUDA-event time "
                             "(FP64-equivalent rate); peak = FP64 directed add/mul instruction rate measured by "
                             "this bench on this GPU (MEASURED_PEAKS.json holds no FP64 figure).  The FP32 pass "
                             "settles ~99% of the boxes' criteria with FP32 enclosures of the FP64 values (same "
                             "decisions), so a frac above 1 is work the FP64 pipe did not have to do, not an "
                             "error; the pass itself is bound by instruction issue (divergent branchy criteria, "
                             "instruction-cache misses: profiles/).  traffic = ncu DRAM bytes per full-size pass"},
        "gpu_launches": int(launches_per_step * args.steps),
        "clocks": ck,
        "e2e": e2e,
    }
    if ws == 1 and not args.no_proof:
        line["proof"] = proof_comparison(prover)
        line["sb_proof"] = sb_proof_run(prover)
        line["sb_forms"] = sb_forms(prover)
        line["near_critical"] = near_critical_run(prover)
    if ws == 1 and not args.no_cpu:
        line["cpu_baseline"] = cpu_baseline(args.cpu_sample)
    prover.close()
    print(json.dumps(line), flush=True)


def proof_comparison(prover):
    """Wall time of the tight proof's initial pass on the small plain-method
    workload (lambda in [1, 1.1] in 256 pieces, r1 in 64, r2..r4 in 128
    each) in three forms, all with identical criticals:
      plain    -- every criterion re-evaluated in every cell, the reference's
                  leaf order;
      batched  -- criteria prepared once per parent cell, compacted stages;
      learned  -- batched, with the leaf criteria ordered per r3 cell by the
                  network, trained first (by the library's kernels) on
                  records from this workload's own plain-order cells."""
    import circlecover_gb300 as cg
    from circlecover_gb300 import learn
    from circlecover_gb300 import workloads as W
    root = W.tight_root(1.0, 1.1)
    grid = cg.make_grid(256, (64, 128, 128, 128))
    out = {"workload": "tight proof, initial pass: lambda [1,1.1] x 256, r1 x 64, r2..r4 x 128"}
    prover.tight_find_critical_intervals(W.tight_root(1.0, 1.0001), cg.make_grid(2, (8, 8, 8, 8)))  # buffers
    t0 = time.perf_counter()
    prover.mlp_init(3)
    rec, ncells = learn.proof_records(prover, root, grid, per_cell=16)
    hist = learn.train(prover, rec, epochs=4, batch=8192)
    train_s = time.perf_counter() - t0
    rep = learn.prediction_report(learn.predict(prover, rec), rec.labels_np)
    res = {}
    for name, kw in (("batched", {}), ("learned", {"learned": True}), ("plain", {"plain": True})):
        t0 = time.perf_counter()
        crit, st = prover.tight_find_critical_intervals(root, grid, **kw)
        res[name] = (time.perf_counter() - t0, crit, st)
    bt, bc, bs = res["batched"]
    keys = ("gen_sizes", "leaf_evals", "trapped_leaves")
    same = all(np.array_equal(r[1].view(np.uint64), bc.view(np.uint64)) and all(r[2][k] == bs[k] for k in keys)
               for r in res.values())
    out.update({"plain_s": res["plain"][0], "batched_s": bt, "learned_s": res["learned"][0],
                "speedup_batched": res["plain"][0] / bt, "speedup_learned": res["plain"][0] / res["learned"][0],
                "leaves": bs["leaf_evals"], "criticals": len(bc), "identical_criticals": bool(same),
                "identical_trace_plain_batched": bool(res["plain"][2]["digest"] == bs["digest"]),
                "training": {"cells_logged": ncells, "records": rec.n, "seconds": train_s, "loss": hist,
                             "error_rate_per_output": rep["error_rate_per_output"]},
                "leaf_outcomes": {k: res[k][2]["counts"][3][:7] for k in res}})
    return out


def near_critical_run(prover, n=1 << 22):
    """Near-critical stress: 2^22 boxes, 90 % with total weight within 1e-4
    (relative) of the critical weight, 10 % drawn as the microbench.  Verdict
    masks of all six criteria (boxes/s, device-resident, CUDA events on the
    launching stream), and the first-success evaluation in the plain order
    and with the trained network's choice first (same decisions)."""
    import torch
    from circlecover_gb300 import learn
    from circlecover_gb300 import workloads as W
    boxes = W.tight_near_critical(n, seed=5)
    soa = torch.from_numpy(W.to_soa(boxes)).cuda()
    masks = torch.empty(n, dtype=torch.int32, device="cuda")
    stream = torch.cuda.Stream()
    torch.cuda.synchronize()
    for _ in range(3):
        prover.tight_eval_device(soa.data_ptr(), n, masks.data_ptr(), stream.cuda_stream)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    steps = 5
    for _ in range(steps):
        prover.tight_eval_device(soa.data_ptr(), n, masks.data_ptr(), stream.cuda_stream)
    e1.record(stream)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / steps
    m = masks.cpu().numpy().view(np.uint32)
    prover.mlp_init(5)
    train_rec = learn.Records(prover, W.tight_near_critical(1 << 20, seed=77))
    learn.train(prover, train_rec, epochs=4, batch=8192)
    rec = learn.Records(prover, boxes)
    cmp = learn.compare_orders(prover, rec)
    cmp.pop("outcomes_plain")
    cmp.pop("outcomes_learned")
    return {"workload": "near-critical stress: 2^22 boxes, 90% within 1e-4 of the critical weight",
            "masks_boxes_per_s": n / (ms * 1e-3), "ms": ms,
            "gaps_certified_share": float(((m >> 5) & 1).mean()),
            "critical_share": float(((m & 0x7F) == 0).mean()), "first_success": cmp}


SB_SLICE = dict(la=(1.0, 1.0 + 1.5 * 2 / 256), grid=(2, (32, 32, 64, 64, 64, 64)))


def sb_proof_run(prover, warm=True):
    """The size-bound proof on a slice of the reference's own initial pass:
    lambda over two of its 256 pieces of [1, 2.5], r1 and r2 in 32 pieces
    (the reference: 128), r3..r6 in 64 pieces (as the reference), every
    squared radius in [0, 9/64]; one pass, no refinement generation."""
    import circlecover_gb300 as cg
    from circlecover_gb300 import workloads as W
    root = W.sb_root(*SB_SLICE["la"])
    la_n, rn = SB_SLICE["grid"]
    if warm:  # buffers are allocated on the first call
        prover.sb_find_critical_intervals(root, cg.make_sb_grid(1, (2, 2, 2, 2, 2, 2)))
    t0 = time.perf_counter()
    crit, flags, st = prover.sb_find_critical_intervals(root, cg.make_sb_grid(la_n, rn))
    dt = time.perf_counter() - t0
    return {"workload": "size-bound proof, initial pass: lambda [1, 1+3/256] x 2, r1 x 32, r2 x 32, r3..r6 x 64",
            "seconds": dt, "leaves": st["leaf_evals"], "leaves_per_s": st["leaf_evals"] / dt,
            "criticals": int(len(crit)), "trapped": int(flags.sum()), "kernel_launches": st["kernel_launches"],
            "leaf_outcomes": st["leaf_counts"], "digest": st["digest"],
            "fp32_prefilter": {"decided_empty": st["fp32_decided"],
                               "decided_share": st["fp32_decided"] / max(1, st["leaf_evals"]),
                               "widening_R_mean": st["widening_mean"], "widening_R_max": st["widening_max"],
                               "widening_samples": st["widening_samples"]}}


def sb_forms(prover):
    """The size-bound proof in its three forms on a smaller workload (lambda
    [1, 1.1] x 8, r1 x 32, r2 x 32, r3..r6 x 16): plain (one thread runs a
    leaf's whole cascade, as the reference's kernel), batched without the
    FP32 pre-filter, batched with it; identical criticals and traces."""
    import circlecover_gb300 as cg
    from circlecover_gb300 import workloads as W
    root = W.sb_root(1.0, 1.1)
    grid = cg.make_sb_grid(8, (32, 32, 16, 16, 16, 16))
    res = {}
    for name, kw in (("batched", {}), ("batched_no_fp32", {"fp32": False}), ("plain", {"plain": True})):
        prover.sb_find_critical_intervals(root, cg.make_sb_grid(1, (2, 2, 2, 2, 2, 2)), **kw)
        t0 = time.perf_counter()
        crit, flags, st = prover.sb_find_critical_intervals(root, grid, **kw)
        res[name] = (time.perf_counter() - t0, crit, flags, st)
    keys = ("task_counts", "cell_counts", "leaf_counts", "digest", "leaf_evals")
    b = res["batched"]
    same = all(np.array_equal(r[1].view(np.uint64), b[1].view(np.uint64)) and np.array_equal(r[2], b[2])
               and all(r[3][k] == b[3][k] for k in keys) for r in res.values())
    return {"workload": "size-bound proof, initial pass: lambda [1,1.1] x 8, r1 x 32, r2 x 32, r3..r6 x 16",
            "leaves": b[3]["leaf_evals"], "batched_s": b[0], "batched_no_fp32_s": res["batched_no_fp32"][0],
            "plain_s": res["plain"][0], "speedup_vs_plain": res["plain"][0] / b[0], "identical": bool(same)}


def ctypes_peak(prover):
    import ctypes
    lib = prover.lib
    lib.cc_selftest_fp64_peak.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.POINTER(ctypes.c_double)]
    v = ctypes.c_double()
    rc = lib.cc_selftest_fp64_peak(prover.h, 0, ctypes.byref(v))
    if rc != 0:
        return float("nan")
    return v.value


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--log2n", type=int, default=24)
    ap.add_argument("--cpu-sample", type=int, default=1 << 23)
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-proof", action="store_true")
    ap.add_argument("--no-autotune", action="store_true")
    ap.add_argument("--workload", default="tight_eval", choices=["tight_eval", "sb_proof", "sb_forms", "tight_proof"])
    args = ap.parse_args()
    ws, rank, local = dist_env()
    if args.workload == "tight_proof":  # the tight proof forms alone (for profiling)
        import __graft_entry__
        __graft_entry__.build()
        import circlecover_gb300 as cg
        with cg.Prover(local) as prover:
            r = proof_comparison(prover)
            if rank == 0:
                print(json.dumps(r), flush=True)
        return
    if args.workload == "sb_forms":  # the smaller size-bound workload in its three forms (for profiling)
        import __graft_entry__
        __graft_entry__.build()
        import circlecover_gb300 as cg
        with cg.Prover(local) as prover:
            for i in range(args.warmup + args.steps):
                r = sb_forms(prover)
                if i >= args.warmup and rank == 0:
                    print(json.dumps(r), flush=True)
        return
    if args.workload == "sb_proof":  # the size-bound proof slice alone (for profiling)
        import __graft_entry__
        __graft_entry__.build()
        import circlecover_gb300 as cg
        with cg.Prover(local) as prover:
            for i in range(args.warmup + args.steps):
                r = sb_proof_run(prover, warm=(i == 0))
                if i >= args.warmup and rank == 0:
                    print(json.dumps(r), flush=True)
        return
    if args.impl == "reference":
        run_reference(args, ws, rank)
        return
    import __graft_entry__
    __graft_entry__.build()
    run_ours(args, ws, rank, local)


if __name__ == "__main__":
    main()
