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
stream), in the certified form: every verdict the FP32 pre-filter decides
"true" is checked again in FP64 (`certification` reports the uncertified
FP32 form and the cost); `e2e` = the same through the host entry point
cc_tight_eval with host buffers (host->device copy of the boxes and
device->host copy of the masks in the timed region); `roofline` per pass
against the instruction rates the library's probe measures on this GPU;
`proof` = the full tight_rectangle proof (the reference's root and schedule)
in its plain, batched and learned forms.  --impl reference times the CPU
implementation of the criteria on the host cores (the reference's own code
where it was built here, otherwise the oracle's port of it) on the same
workload.  --workload config1 runs the small plain-method proof in the three
forms instead.
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
    for the host; first 2**16 boxes of the 2**24-box set), and the golden
    masks of those boxes."""
    z = np.load(os.path.join(ROOT, "tests", "golden", "tight_bench_ops.npz"))
    return float(z["ops"].astype(np.float64).mean()), z["masks"]


PROFILE = os.path.join(ROOT, "profiles", "tight_eval_microbench_2e24.md")


def profile_per_box():
    """Per-box counts of each evaluation pass from the committed ncu summary
    (lines `per_box[<pass>].<metric>: value`, measured on a 2^21-box sample of
    this workload): warp instructions, thread instructions, FP64 and FP32
    thread instructions, DRAM bytes.  Counts grow with the number of boxes."""
    out = {}
    if not os.path.exists(PROFILE):
        return out
    for line in open(PROFILE):
        if not line.startswith("per_box["):
            continue
        key, val = line.split(":", 1)
        name, metric = key[len("per_box["):].split("].", 1)
        try:
            out.setdefault(name, {})[metric.strip()] = float(val)
        except ValueError:
            pass
    return out


def hbm_view(traffic_bytes, ms):
    """The dominant pass against the HBM roofline: its DRAM traffic (ncu bytes
    per box x boxes) per second of its live time, as a fraction of the copy
    bandwidth measured on this machine (MEASURED_PEAKS.json, when present)."""
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    peak = None
    if os.path.exists(path):
        try:
            peak = float(json.load(open(path))["hbm_gbs"])
        except (ValueError, KeyError, OSError):
            peak = None
    if not traffic_bytes or not ms or ms <= 0:
        return None
    achieved = traffic_bytes / (ms * 1e-3) / 1e9
    return {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
            "frac": achieved / peak if peak else None, "source": "MEASURED_PEAKS.json hbm_gbs (measured copy)"}


def peaks(prover):
    """Instruction-throughput ceilings measured on this GPU by the library's
    probe (cc_selftest_peak): FP64 directed add/mul, FP32 directed add/mul and
    FP32 FMA thread instructions per second; the FP32 FMA rate / 32 is the
    warp-instruction issue rate (one FMA warp instruction per cycle per SM
    sub-partition)."""
    import ctypes
    lib = prover.lib
    lib.cc_selftest_peak.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.POINTER(ctypes.c_double)]
    out = {}
    for name, kind in (("fp64", 0), ("fp64_fma", 1), ("fp32", 2), ("fp32_fma", 3)):
        v = ctypes.c_double()
        rc = lib.cc_selftest_peak(prover.h, kind, ctypes.byref(v))
        out[name] = v.value if rc == 0 else float("nan")
    out["issue"] = out["fp32_fma"] / 32.0
    return out


FP64_PASSES = ("k_eval_main", "k_eval_cover", "k_eval_gaps", "k_eval_cert", "k_eval_repair")


def pass_rooflines(stage_ms, n, pk, per_box):
    """Per-pass roofline from the live pass times: the FP32 pass against the
    warp-instruction issue rate, the FP64 passes against the FP64 pipe in
    useful (active-lane) operations; DRAM traffic per launch alongside."""
    import circlecover_gb300 as cg
    res = {}
    for i, name in enumerate(cg.EVAL_PASSES):
        ms = float(stage_ms[i])
        d = per_box.get(name, {})
        r = {"ms": ms}
        if d and ms > 0:
            sec = ms * 1e-3
            warp = d.get("warp_inst", 0.0) * n
            thr = d.get("thread_inst", 0.0) * n
            f64 = d.get("fp64_inst", 0.0) * n
            r.update({"warp_inst_per_s": warp / sec, "issue_frac": warp / sec / pk["issue"],
                      "lanes_per_inst": thr / warp if warp else None,
                      "fp64_ops_per_s": f64 / sec, "fp64_useful_frac": f64 / sec / pk["fp64"],
                      "traffic_bytes": d.get("dram_bytes", 0.0) * n})
            r["bound"] = "fp64" if name in FP64_PASSES else "issue"
        res[name] = r
    return res


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
    # one core on a sixteenth of the sample
    n1 = max(4096, n_sample // 16)
    t0 = time.perf_counter()
    impl.tight_eval(boxes[:n1], threads=1)
    dt1 = time.perf_counter() - t0
    return {"value": n_sample / dt, "unit": UNIT, "cores": cores, "kind": kind,
            "sample": "first %d boxes of the 2^24-box microbench (seed 1), %d threads, %.2f s" % (n_sample, cores, dt),
            "single_core": {"value": n1 / dt1, "unit": UNIT, "cores": 1,
                            "sample": "first %d boxes, 1 thread, %.2f s" % (n1, dt1)}}


def cpu_variants(n_sample=1 << 16, seed=1):
    """The CPU implementations side by side on the first n_sample boxes of the
    microbench: the reference's own criteria built for the host with the
    error-free-transform rounding layer and with fesetround (where the
    reference sources are present), and the oracle's port of them, each on
    one thread and on all host threads (boxes/s; masks checked equal)."""
    import ctypes
    from circlecover_gb300 import workloads as W
    from oracle import oracle as O
    from oracle import build as OB
    O.ensure_built()
    cores = os.cpu_count() or 1
    boxes = W.tight_microbench(n_sample, seed=seed)
    impls = [("port", O.Port())]
    if O.ref_available():
        impls.insert(0, ("reference_eft", O.Ref()))
        fe = OB.build_ref_fenv()
        if fe:
            impls.insert(1, ("reference_fesetround", O.Ref(fe)))
    out = {"boxes": n_sample, "cores": cores, "cpu": _cpu_model(), "results": {}}
    want = None
    for name, impl in impls:
        row = {}
        for threads in (1, cores):
            sample = boxes if threads > 1 else boxes[: max(1024, n_sample // 8)]
            impl.tight_eval(sample[:1024], threads=threads)
            t0 = time.perf_counter()
            m = impl.tight_eval(sample, threads=threads)
            dt = time.perf_counter() - t0
            row["threads_%d" % threads] = len(sample) / dt
            if threads > 1:
                if want is None:
                    want = m
                row["masks_equal"] = bool(np.array_equal(m, want))
        out["results"][name] = row
    return out


def _cpu_model():
    try:
        for line in open("/proc/cpuinfo"):
            if line.lower().startswith(("model name", "cpu part")):
                return line.split(":", 1)[1].strip()
    except OSError:
        pass
    return None


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

    def timed(steps):
        """mean ms per step over `steps` steps (CUDA events on the stream),
        max over ranks"""
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(steps):
            step()
        e1.record(stream)
        barrier()
        ms = e0.elapsed_time(e1) / steps
        if ws > 1:
            t = torch.tensor([ms], device="cuda", dtype=torch.float64)
            torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
            ms = float(t.item())
        return ms

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
    # the uncertified FP32 form (opt-in, measurement only), timed first
    prover.set_eval_certify(False)
    for _ in range(args.warmup):
        step()
    barrier()
    ms_fp32_only = timed(args.steps)
    prover.set_eval_certify(True)
    # the product: every FP32-decided "true" verdict certified in FP64
    for _ in range(args.warmup):
        step()
    barrier()
    launches_per_step = prover.last_launch_count
    cert = prover.eval_cert_counts()
    queues = prover.eval_counts()
    clocks = ClockSampler(local)
    clocks.start()
    ms = timed(args.steps)
    ck = clocks.stop()
    value = ws * n / (ms * 1e-3)
    # per-pass CUDA events (recorded by the library on the same stream), in
    # separate steps so that the headline steps run as one graph launch each
    prover.set_stage_timing(True)
    stage_ms = np.zeros(len(cg.EVAL_PASSES))
    for _ in range(args.steps):
        step()
        stage_ms += np.array(prover.stage_times())
    prover.set_stage_timing(False)
    stage_ms /= args.steps

    # correctness of the timed output: the sampled boxes' masks equal the
    # reference's (golden) masks
    ops_per_box, ref_masks = algorithmic_ops_per_box()
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
    pk = peaks(prover)
    per_box = profile_per_box()
    passes = pass_rooflines(stage_ms, n, pk, per_box)
    dom = cg.EVAL_PASSES[int(np.argmax(stage_ms))]
    dp = passes[dom]
    if dp.get("bound") == "fp64":
        roof = {"bound": "fp64", "achieved": dp["fp64_ops_per_s"] / 1e12, "peak": pk["fp64"] / 1e12,
                "unit": "T FP64 thread-ops/s (active lanes only)", "frac": dp["fp64_useful_frac"],
                "probe": "cc_selftest_peak kind 0 (FP64 directed add/mul chains)"}
    elif dp.get("bound") == "issue":
        roof = {"bound": "issue", "achieved": dp["warp_inst_per_s"] / 1e9, "peak": pk["issue"] / 1e9,
                "unit": "G warp-instructions/s", "frac": dp["issue_frac"],
                "probe": "cc_selftest_peak kind 3 (FP32 FMA chains) / 32"}
    else:
        roof = {"bound": None, "achieved": None, "peak": None, "unit": None, "frac": None,
                "probe": "no ncu per-box counts committed for this pass"}
    step_ref_ops = ops_per_box * n / (ms * 1e-3)
    roof.update({
        "kernel": dom, "traffic": dp.get("traffic_bytes"), "algorithmic_bytes": 84 * n,
        "hbm": hbm_view(dp.get("traffic_bytes"), dp.get("ms")),
        "lanes_per_inst": dp.get("lanes_per_inst"), "passes": passes,
        "peaks": {k: v / 1e12 for k, v in pk.items()}, "peaks_unit": "T thread-instructions/s (issue: T warp-inst/s)",
        "fp64_equivalent": {"ref_fp64_ops_per_box": ops_per_box, "rate": step_ref_ops / 1e12,
                            "unit": "T reference-FP64-ops/s", "vs_fp64_peak": step_ref_ops / pk["fp64"],
                            "note": "the reference's FP64 directed-rounding operations per box (shim-counted) "
                                    "x boxes / step time: FP64 work the reference does per box, most of "
                                    "which this build decides on FP32 enclosures; not a pipe utilisation"},
        "note": "achieved = executed instructions per box (ncu, profiles/tight_eval_microbench_2e24.md, "
                "2^21-box sample) x boxes / the pass's live CUDA-event time; peak = this GPU's "
                "instruction rate measured by the library's probe at bench time; traffic = ncu DRAM "
                "bytes per box x boxes; algorithmic_bytes = 80 B in + 4 B out per box"})
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": ms, "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded, platform-independent generator)",
        "config": {"workload": "tight criteria microbench: 2^24 boxes per GPU, lambda~U[1,4], log-uniform widths "
                               "2^-20..2^-4, total weight critical*(1+eps), eps log-uniform 1e-6..1e-1",
                   "boxes_per_gpu": n, "l2_flush": "not needed: inputs (%.2f GB) exceed L2" % (n * 80 / 1e9),
                   "layout": "SoA, 10 x n float64", "autotune": tune,
                   "form": "certified: every FP32-decided true verdict re-checked in FP64"},
        "verified_vs_reference_masks": verified,
        "certification": {"counts": cert, "queues": queues,
                          "fp32_uncertified": {"ms_per_step": ms_fp32_only, "value": ws * n / (ms_fp32_only * 1e-3)},
                          "cost": ms / ms_fp32_only},
        "roofline": roof,
        "gpu_launches": int(launches_per_step * args.steps),
        "clocks": ck,
        "e2e": e2e,
    }
    if ws == 1 and not args.no_proof:
        line["proof"] = proof_comparison(prover)
        line["sb_proof"] = sb_proof_run(prover)
        line["sb_forms"] = sb_forms(prover)
        line["near_critical"] = near_critical_run(prover)
        line["near_critical"]["refinement"] = near_critical_refinement()
        line["small_batch"] = small_batch_run(prover)
    if ws == 1 and not args.no_cpu:
        line["cpu_baseline"] = cpu_baseline(args.cpu_sample)
    prover.close()
    print(json.dumps(line), flush=True)


# the reference's schedule (tight_rectangle.cu:44-58): initial splits, then
# eleven refinement generations with these lambda splits and r splits
TIGHT_GENS = (1, 2, 2, 2, 2, 1, 2, 1, 2, 1, 2)
TIGHT_R_GEN = (128, 128, 128, 64)
PROOFS = {
    # the full tight_rectangle proof: lambda in [1, 2.0898841580413818342]
    # (tight_rectangle.cu:461-464), 256 x 128^4 initial splits
    "full": ("tight proof, full (reference schedule): lambda [1, 2.0899] x 256, r1..r4 x 128, 11 generations "
             "(lambda x 1 or 2, r 128^3 x 64)", (1.0, None), (256, (128, 128, 128, 128))),
    # the plain-method workload: lambda in [1, 1.1], r1 in 64 pieces
    "config1": ("tight proof, small plain-method workload: lambda [1, 1.1] x 256, r1 x 64, r2..r4 x 128, "
                "refinement schedule of the reference", (1.0, 1.1), (256, (64, 128, 128, 128))),
}


def proof_comparison(prover, which="full", n_microbench_records=10_000_000):
    """Wall time of a whole tight proof in three forms, all with identical
    criticals, generation sizes and leaf counts:
      plain    -- every criterion re-evaluated in every cell, the reference's
                  leaf order, FP64 only;
      batched  -- criteria prepared once per parent cell, compacted stages,
                  leaf criteria FP32-first with every FP32 "true" certified
                  in FP64;
      learned  -- batched, with the leaf criteria ordered per r3 cell by the
                  network, trained first (by the library's kernels) on
                  records of the initial pass's plain-order cells."""
    import circlecover_gb300 as cg
    from circlecover_gb300 import learn
    from circlecover_gb300 import workloads as W
    desc, (la_lo, la_hi), (la0, r0) = PROOFS[which]
    root = W.tight_root(la_lo, la_hi if la_hi is not None else W.TIGHT_LAMBDA_MAX)
    grid = cg.make_grid(la0, r0, TIGHT_GENS, TIGHT_R_GEN)
    out = {"workload": desc}
    prover.tight_find_critical_intervals(W.tight_root(1.0, 1.0001), cg.make_grid(2, (8, 8, 8, 8)))  # buffers
    t0 = time.perf_counter()
    prover.mlp_init(3)
    rec, ncells = learn.proof_records(prover, root, cg.make_grid(la0, r0), per_cell=16)
    hist = learn.train(prover, rec, epochs=4, batch=8192)
    train_s = time.perf_counter() - t0
    logits_proof = learn.predict(prover, rec)
    rep = learn.prediction_report(logits_proof, rec.labels_np)
    res = {}
    for name, kw in (("batched", {}), ("learned", {"learned": True}), ("plain", {"plain": True})):
        t0 = time.perf_counter()
        crit, st = prover.tight_find_critical_intervals(root, grid, **kw)
        res[name] = (time.perf_counter() - t0, crit, st)
    # the same network trained instead on ~1e7 records of the criteria
    # microbench (boxes labelled by their verdict masks), driving the same proof
    t0 = time.perf_counter()
    prover.mlp_init(4)
    rec_mb = learn.Records(prover, W.tight_microbench(n_microbench_records, seed=44))
    hist_mb = learn.train(prover, rec_mb, epochs=4, batch=8192)
    train_mb_s = time.perf_counter() - t0
    rep_mb = learn.prediction_report(learn.predict(prover, rec), rec.labels_np)  # on the proof's own records
    del rec_mb
    t0 = time.perf_counter()
    crit, st = prover.tight_find_critical_intervals(root, grid, learned=True)
    res["learned_microbench"] = (time.perf_counter() - t0, crit, st)
    bt, bc, bs = res["batched"]
    keys = ("gen_sizes", "leaf_evals", "trapped_leaves")
    same = all(np.array_equal(r[1].view(np.uint64), bc.view(np.uint64)) and all(r[2][k] == bs[k] for k in keys)
               for r in res.values())
    split_pred = logits_proof[:, 6] > 0
    out.update({"plain_s": res["plain"][0], "batched_s": bt, "learned_s": res["learned"][0],
                "speedup_batched": res["plain"][0] / bt, "speedup_learned": res["plain"][0] / res["learned"][0],
                "learned_microbench_s": res["learned_microbench"][0],
                "speedup_learned_microbench": res["plain"][0] / res["learned_microbench"][0],
                "training_microbench": {"records": n_microbench_records, "seconds": train_mb_s, "loss": hist_mb,
                                        "error_rate_per_output_on_proof_records": rep_mb["error_rate_per_output"]},
                "split_output": {"error_rate": rep["split_error_rate"],
                                 "predicted_split_share": float(split_pred.mean()), "acted_on": False},
                "leaves": bs["leaf_evals"], "criticals": len(bc), "gen_sizes": bs["gen_sizes"],
                "identical_criticals": bool(same),
                "identical_trace_plain_batched": bool(res["plain"][2]["digest"] == bs["digest"]),
                "digest": bs["digest"],
                "training": {"cells_logged": ncells, "records": rec.n, "seconds": train_s, "loss": hist,
                             "error_rate_per_output": rep["error_rate_per_output"]},
                "leaf_outcomes": {k: res[k][2]["counts"][3][:7] for k in res},
                "fp32_first": {k: res[k][2]["fp32_first"] for k in res},
                "cert_failures": {k: res[k][2]["cert_failures"] for k in res},
                "kernel_launches": {k: res[k][2]["kernel_launches"] for k in res}})
    return out


def small_batch_run(prover, n=1 << 16, reps=20):
    """Batches of 65,536 boxes (the largest the allocation-free entry takes):
    cc_tight_eval_device (handle-owned queues, recorded calls, graph replay)
    next to cc_tight_eval_device_static (a fixed array, no recorded calls:
    the one-kernel FP32 pass), CUDA events on one stream; same masks."""
    import torch
    from circlecover_gb300 import workloads as W
    boxes = W.tight_microbench(n, seed=1)
    soa = torch.from_numpy(W.to_soa(boxes)).cuda()
    m_dev = torch.empty(n, dtype=torch.int32, device="cuda")
    m_st = torch.empty(n, dtype=torch.int32, device="cuda")
    stream = torch.cuda.Stream()
    torch.cuda.synchronize()
    out = {"boxes": n}
    for name, call, m in (("device", prover.tight_eval_device, m_dev),
                          ("static", prover.tight_eval_device_static, m_st)):
        for _ in range(3):
            call(soa.data_ptr(), n, m.data_ptr(), stream.cuda_stream)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(reps):
            call(soa.data_ptr(), n, m.data_ptr(), stream.cuda_stream)
        e1.record(stream)
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1) / reps
        out[name] = {"ms": ms, "boxes_per_s": n / (ms * 1e-3)}
    out["same_masks"] = bool(torch.equal(m_dev, m_st))
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


def proof_batched_only(prover, which="full"):
    """The batched, certified form of a tight proof alone (for launch lists
    and profiles of the proof's kernels)."""
    import circlecover_gb300 as cg
    from circlecover_gb300 import workloads as W
    desc, (la_lo, la_hi), (la0, r0) = PROOFS[which]
    root = W.tight_root(la_lo, la_hi if la_hi is not None else W.TIGHT_LAMBDA_MAX)
    prover.tight_find_critical_intervals(W.tight_root(1.0, 1.0001), cg.make_grid(2, (8, 8, 8, 8)))  # buffers
    t0 = time.perf_counter()
    crit, st = prover.tight_find_critical_intervals(root, cg.make_grid(la0, r0, TIGHT_GENS, TIGHT_R_GEN))
    return {"workload": desc, "form": "batched", "seconds": time.perf_counter() - t0, "leaves": st["leaf_evals"],
            "criticals": len(crit), "gen_sizes": st["gen_sizes"], "digest": st["digest"],
            "fp32_first": st["fp32_first"], "cert_failures": st["cert_failures"],
            "kernel_launches": st["kernel_launches"]}


def _refine_summary(crit, flags, st):
    live = np.array(st["live"], dtype=np.float64)
    occ = {k: [round(v / max(1.0, l), 5) for v, l in zip(st[k], live)]
           for k in ("fp64_boxes", "cover_jobs", "gaps_jobs", "cert_jobs")}
    out = {"seconds": st["seconds"], "depths_run": st["depths_run"], "stopped_at_cap": st["stopped_at_cap"],
           "boxes_evaluated": int(live.sum()), "boxes_per_s": float(live.sum() / st["seconds"]),
           "criticals": int(len(crit)), "trapped": int((flags == 1).sum()), "cut": int((flags == 3).sum()),
           "live": st["live"],
           "decided": st["decided"], "ms": [round(x, 3) for x in st["ms"]],
           "kernel_launches": st["kernel_launches"]}
    if st["order"] == 0:
        out["queue_share_of_live"] = occ
    else:
        steps, wmax = np.array(st["steps"], dtype=np.float64), np.array(st["warp_max_steps"], dtype=np.float64)
        out["mean_steps"] = float(steps.sum() / max(1.0, live.sum()))
        out["lane_share_per_depth"] = [round(a / max(1.0, 32 * b), 4) for a, b in zip(steps, wmax)]
        out["lane_share"] = float(steps.sum() / max(1.0, 32 * wmax.sum()))
    return out


def near_critical_refinement(n=1 << 22, max_depth=32, max_live=1 << 25, n_orders=1 << 18, orders_live=1 << 23):
    """Config 5: the near-critical boxes refined by bisection to depth 32
    (cc_tight_refine).  The undecided population about doubles per level
    (the boxes around the critical configurations are never certified), so
    a level carries at most max_live boxes on: the first ones in level order,
    the others are kept as criticals (flag 3, `cut`).  On a fresh handle: the
    certified evaluation of all criteria per level with the default pass
    settings, then with the passes tuned on the near-critical boxes
    themselves (same criticals); per depth the live and decided boxes, the
    device time and the queue occupancy.  On the first n_orders boxes (cap
    orders_live): the same refinement by first-success evaluation in the
    plain order and with the trained network's choice first, with the share
    of lanes working per warp (load balance)."""
    import torch
    import circlecover_gb300 as cg
    from circlecover_gb300 import learn
    from circlecover_gb300 import workloads as W
    boxes = W.tight_near_critical(n, seed=5)
    res = {"workload": "near-critical stress refinement: 2^22 boxes, 90%% within 1e-4 of the critical weight, "
                       "bisection (lambda, r1..r4 in turn) to depth %d, at most %d live boxes per level (the "
                       "first in level order; the rest kept as cut criticals)" % (max_depth, max_live)}

    def same(a, b):  # criticals, flags and level sizes (the output order is deterministic)
        return bool(len(a[0]) == len(b[0]) and np.array_equal(a[0].view(np.uint64), b[0].view(np.uint64))
                    and np.array_equal(a[1], b[1]) and a[2]["live"] == b[2]["live"])

    with cg.Prover(0) as p:
        p.tight_refine(boxes[:4096], max_depth=4)  # buffers, kernels
        r_def = p.tight_refine(boxes, max_depth, max_live)
        m = 1 << 22
        soa = torch.from_numpy(W.to_soa(boxes[:m])).cuda()
        msk = torch.empty(m, dtype=torch.int32, device="cuda")
        torch.cuda.synchronize()
        tune = p.autotune_eval(soa.data_ptr(), m, msk.data_ptr())
        del soa, msk
        r_tuned = p.tight_refine(boxes, max_depth, max_live)
        res["default"] = _refine_summary(*r_def)
        res["autotuned"] = _refine_summary(*r_tuned)
        res["autotune"] = tune
        res["identical_default_autotuned"] = same(r_def, r_tuned)
        sub = boxes[:n_orders]
        p.mlp_init(5)
        learn.train(p, learn.Records(p, W.tight_near_critical(1 << 20, seed=77)), epochs=4, batch=8192)
        orders = {}
        for order in ("masks", "first_plain", "first_learned"):
            p.tight_refine(sub[:2048], 2, order=order)
            orders[order] = p.tight_refine(sub, max_depth, orders_live, order=order)
        res["orders"] = {"boxes": n_orders, **{k: _refine_summary(*v) for k, v in orders.items()},
                         "identical_criticals": all(same(v, orders["masks"]) for v in orders.values())}
    return res


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
                               "widening_samples": st["widening_samples"]},
            "certification": {"fp32_true_certified": st["fp32_certified"],
                              "empty_anchors_certified": st["empty_anchors"],
                              "failures": st["cert_failures"]}}


SB_FULL = {
    # the reference's own size-bound proof (rectangle_size_bound.cu:36-62,
    # 312-382): lambda in [1, 2.5], 256 x 128 x 128 tasks, r3..r6 in 64, one
    # refinement generation (lambda x 64, r 32,32,16,16,16,32)
    "sb_reference": ("size-bound proof, the reference's own: lambda [1, 2.5] x 256, r1 x 128, r2 x 128, r3..r6 x 64, "
                     "1 refinement generation (lambda x 64, r 32,32,16,16,16,32)", (1.0, 2.5),
                     (256, (128, 128, 64, 64, 64, 64), 64, (32, 32, 16, 16, 16, 32), 1)),
    # the size-bound run over lambda in [1, 8]: 1024 lambda pieces x 256 r1
    # pieces (r2 and r3..r6 as the reference), refinement generations with
    # the reference's refinement splits while criticals remain, at most 24
    "config3": ("size-bound proof, lambda [1, 8] x 1024, r1 x 256, r2 x 128, r3..r6 x 64, up to 24 refinement "
                "generations (lambda x 64, r 32,32,16,16,16,32)", (1.0, 8.0),
                (1024, (256, 128, 64, 64, 64, 64), 64, (32, 32, 16, 16, 16, 32), 24)),
}


def sb_full_run(prover, which):
    """A whole size-bound proof (SB_FULL) in the batched, certified form."""
    import circlecover_gb300 as cg
    from circlecover_gb300 import workloads as W
    desc, (la_lo, la_hi), (la0, r0, lag, rg, gens) = SB_FULL[which]
    prover.sb_find_critical_intervals(W.sb_root(1.0, 1.01), cg.make_sb_grid(1, (2, 2, 2, 2, 2, 2)))  # buffers
    t0 = time.perf_counter()
    crit, flags, st = prover.sb_find_critical_intervals(W.sb_root(la_lo, la_hi), cg.make_sb_grid(la0, r0, lag, rg, gens))
    dt = time.perf_counter() - t0
    return {"workload": desc, "seconds": dt, "leaves": st["leaf_evals"], "leaves_per_s": st["leaf_evals"] / dt,
            "criticals": int(len(crit)), "trapped": int(flags.sum()), "gen_sizes": st["gen_sizes"],
            "task_counts": st["task_counts"], "leaf_outcomes": st["leaf_counts"], "digest": st["digest"],
            "kernel_launches": st["kernel_launches"],
            "fp32_prefilter": {"decided_empty": st["fp32_decided"],
                               "decided_share": st["fp32_decided"] / max(1, st["leaf_evals"]),
                               "widening_R_mean": st["widening_mean"], "widening_R_max": st["widening_max"]},
            "certification": {"fp32_true_certified": st["fp32_certified"],
                              "empty_anchors_certified": st["empty_anchors"], "failures": st["cert_failures"]}}


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
    ap.add_argument("--workload", default="tight_eval",
                    choices=["tight_eval", "sb_proof", "sb_forms", "tight_proof", "config1", "cpu_variants",
                             "sb_reference", "config3", "near_critical", "tight_proof_batched"])
    args = ap.parse_args()
    ws, rank, local = dist_env()
    if args.workload in SB_FULL:  # a whole size-bound proof (minutes)
        import __graft_entry__
        __graft_entry__.build()
        import circlecover_gb300 as cg
        with cg.Prover(local) as prover:
            r = sb_full_run(prover, args.workload)
            if rank == 0:
                print(json.dumps(r), flush=True)
        return
    if args.workload == "near_critical":  # config 5's refinement alone
        import __graft_entry__
        __graft_entry__.build()
        r = near_critical_refinement()
        if rank == 0:
            print(json.dumps(r), flush=True)
        return
    if args.workload == "cpu_variants":  # the CPU implementations side by side (no GPU)
        print(json.dumps(cpu_variants(args.cpu_sample)), flush=True)
        return
    if args.workload == "tight_proof_batched":  # the batched form of the full tight proof alone
        import __graft_entry__
        __graft_entry__.build()
        import circlecover_gb300 as cg
        with cg.Prover(local) as prover:
            r = proof_batched_only(prover)
            if rank == 0:
                print(json.dumps(r), flush=True)
        return
    if args.workload in ("tight_proof", "config1"):  # the tight proof forms alone
        import __graft_entry__
        __graft_entry__.build()
        import circlecover_gb300 as cg
        with cg.Prover(local) as prover:
            r = proof_comparison(prover, "full" if args.workload == "tight_proof" else "config1")
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
