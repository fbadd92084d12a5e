"""circlecover_gb300 -- GB300 (sm_103a) prover for the rectangle-covering-by-
disks proofs of phillip-keldenich/circlecover.

Python host mirror of the C ABI in ``include/circlecover_gb300.h`` (ctypes
over ``_build/libcirclecover_gb300.so``).  The names follow the reference:
``Prover.tight_find_critical_intervals`` is the reference's
``circlecover::tight_rectangle::find_critical_intervals()``
(tight_rectangle/tight_rectangle.cu:458), ``Prover.tight_eval`` evaluates the
criteria declared in tight_rectangle/strategies.cuh:54-87.

There is no CPU fallback: if the CUDA library is missing or no device is
usable, every entry point raises.
"""
import ctypes
import os

import numpy as np

from .workloads import TIGHT_BOX, SB_BOX  # noqa: F401

PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(PKG, "_build", "libcirclecover_gb300.so")

MAX_GEN = 32

# verdict bits (CC_TV_*)
TV_R1, TV_R1R2, TV_R1R2R3, TV_TWO_BY_TWO, TV_R1R2R3_LEAF, TV_GAPS, TV_R_EMPTY = (1 << k for k in range(7))
TV_TRAPPED = 1 << 31

# reference split counts (tight_rectangle.cu:44-58)
REFERENCE_GRID = dict(la_init=256, r_init=(128, 128, 128, 128), gens=(1, 2, 2, 2, 2, 1, 2, 1, 2, 1, 2),
                      r_gen=(128, 128, 128, 64))


# reference split counts of the size-bound proof (rectangle_size_bound.cu:36-62)
REFERENCE_SB_GRID = dict(la_init=256, r_init=(128, 128, 64, 64, 64, 64), la_gen=64, r_gen=(32, 32, 16, 16, 16, 32),
                         gens=1)
SB_LEAF_OUTCOMES = 17
SBT_LEAF_EMPTY, SBT_LEAF_CRITICAL, SBT_LEAF_TRAPPED = 14, 15, 16


class CudaError(RuntimeError):
    pass


class CcIv(ctypes.Structure):
    _fields_ = [("lb", ctypes.c_double), ("ub", ctypes.c_double)]


class CcTightBox(ctypes.Structure):
    _fields_ = [("la", CcIv), ("r", CcIv * 4)]


class CcTightGrid(ctypes.Structure):
    _fields_ = [
        ("la_splits_init", ctypes.c_int),
        ("r_splits_init", ctypes.c_int * 4),
        ("num_generations", ctypes.c_int),
        ("la_splits_gen", ctypes.c_int * MAX_GEN),
        ("r_splits_gen", ctypes.c_int * 4),
    ]


class CcProveStats(ctypes.Structure):
    _fields_ = [
        ("counts", (ctypes.c_uint64 * 8) * 4),
        ("digest", ctypes.c_uint64),
        ("leaf_evals", ctypes.c_uint64),
        ("trapped_leaves", ctypes.c_uint64),
        ("gen_sizes", ctypes.c_uint64 * (MAX_GEN + 1)),
        ("generations_run", ctypes.c_int32),
        ("reserved", ctypes.c_int32),
        ("seconds", ctypes.c_double),
        ("kernel_launches", ctypes.c_uint64),
        ("fp32_first", ctypes.c_uint64 * 4),
        ("cert_failures", ctypes.c_uint64),
    ]


class CcTightSummary(ctypes.Structure):
    """cc_tight_summary_t (Max_distances, tight_rectangle.cu:322-341)."""
    _fields_ = [
        ("have_range_2d", ctypes.c_int32), ("have_range_3d", ctypes.c_int32),
        ("la_range_2d", CcIv), ("la_range_3d", CcIv),
        ("dist_r1_2d", CcIv), ("dist_r1_2d_criticals", CcTightBox * 2),
        ("dist_r2_2d", CcIv), ("dist_r2_2d_criticals", CcTightBox * 2),
        ("lb_h1_2d", ctypes.c_double), ("ub_la_by_S1", ctypes.c_double), ("ub_R3_2d", ctypes.c_double),
        ("dist_r1_3d", CcIv), ("dist_r1_3d_criticals", CcTightBox * 2),
        ("dist_r2_3d", CcIv), ("dist_r2_3d_criticals", CcTightBox * 2),
        ("dist_r3_3d", CcIv), ("dist_r3_3d_criticals", CcTightBox * 2),
        ("ub_R4_3d", ctypes.c_double),
        ("S1", CcIv), ("h2", CcIv), ("S3", CcIv),
        ("pocket_width_3d", ctypes.c_double),
    ]


REFINE_MAX_DEPTH = 48


class CcRefineStats(ctypes.Structure):
    _fields_ = [("live", ctypes.c_uint64 * (REFINE_MAX_DEPTH + 1)),
                ("decided", ctypes.c_uint64 * (REFINE_MAX_DEPTH + 1)),
                ("ms", ctypes.c_float * (REFINE_MAX_DEPTH + 1)),
                ("depths_run", ctypes.c_int32), ("stopped_at_cap", ctypes.c_int32),
                ("seconds", ctypes.c_double), ("kernel_launches", ctypes.c_uint64),
                ("fp64_boxes", ctypes.c_uint64 * (REFINE_MAX_DEPTH + 1)),
                ("cover_jobs", ctypes.c_uint64 * (REFINE_MAX_DEPTH + 1)),
                ("gaps_jobs", ctypes.c_uint64 * (REFINE_MAX_DEPTH + 1)),
                ("cert_jobs", ctypes.c_uint64 * (REFINE_MAX_DEPTH + 1)),
                ("steps", ctypes.c_uint64 * (REFINE_MAX_DEPTH + 1)),
                ("warp_max_steps", ctypes.c_uint64 * (REFINE_MAX_DEPTH + 1)),
                ("cut", ctypes.c_uint64 * (REFINE_MAX_DEPTH + 1)),
                ("order", ctypes.c_int32), ("pad", ctypes.c_int32)]


REFINE_ORDERS = {"masks": 0, "first_plain": 1, "first_learned": 2}


class CcTuneResult(ctypes.Structure):
    _fields_ = [("min_blocks", ctypes.c_int * 4), ("blocks_per_sm", ctypes.c_int * 4), ("ms", ctypes.c_float * 4),
                ("ms_default", ctypes.c_float * 4)]


# the evaluation's passes (cc_last_stage_times order); the first four are
# the ones the autotuner tunes
EVAL_PASSES = ("k_eval_f32", "k_eval_main", "k_eval_cover", "k_eval_gaps", "k_eval_cert", "k_eval_repair")
TUNED_PASSES = EVAL_PASSES[:4]


class CcSbGrid(ctypes.Structure):
    _fields_ = [
        ("la_splits_init", ctypes.c_int),
        ("r_splits_init", ctypes.c_int * 6),
        ("la_splits_gen", ctypes.c_int),
        ("r_splits_gen", ctypes.c_int * 6),
        ("num_generations", ctypes.c_int),
    ]


class CcSbProveStats(ctypes.Structure):
    _fields_ = [
        ("task_counts", ctypes.c_uint64 * 4),
        ("cell_counts", ctypes.c_uint64 * 4),
        ("leaf_counts", ctypes.c_uint64 * SB_LEAF_OUTCOMES),
        ("digest", ctypes.c_uint64),
        ("leaf_evals", ctypes.c_uint64),
        ("trapped_leaves", ctypes.c_uint64),
        ("trapped_shortcuts", ctypes.c_uint64),
        ("gen_sizes", ctypes.c_uint64 * (MAX_GEN + 1)),
        ("generations_run", ctypes.c_int32),
        ("reserved", ctypes.c_int32),
        ("seconds", ctypes.c_double),
        ("kernel_launches", ctypes.c_uint64),
        ("fp32_decided", ctypes.c_uint64),
        ("widening_samples", ctypes.c_uint64),
        ("widening_mean", ctypes.c_double),
        ("widening_max", ctypes.c_double),
        ("fp32_certified", ctypes.c_uint64),
        ("empty_anchors", ctypes.c_uint64),
        ("cert_failures", ctypes.c_uint64),
    ]


def make_sb_grid(la_init, r_init, la_gen=64, r_gen=(32, 32, 16, 16, 16, 32), gens=0):
    """Split counts of the size-bound proof (cc_sb_grid)."""
    g = CcSbGrid()
    g.la_splits_init = la_init
    g.la_splits_gen = la_gen
    for k in range(6):
        g.r_splits_init[k] = r_init[k]
        g.r_splits_gen[k] = r_gen[k]
    g.num_generations = gens
    return g


def sb_stats_to_dict(s):
    return {
        "task_counts": [int(x) for x in s.task_counts],
        "cell_counts": [int(x) for x in s.cell_counts],
        "leaf_counts": [int(x) for x in s.leaf_counts],
        "digest": int(s.digest),
        "leaf_evals": int(s.leaf_evals),
        "trapped_leaves": int(s.trapped_leaves),
        "trapped_shortcuts": int(s.trapped_shortcuts),
        "gen_sizes": [int(s.gen_sizes[g]) for g in range(int(s.generations_run) + 1)],
        "generations_run": int(s.generations_run),
    }


def make_grid(la_init, r_init, gens=(), r_gen=(128, 128, 128, 64)):
    g = CcTightGrid()
    g.la_splits_init = int(la_init)
    for k in range(4):
        g.r_splits_init[k] = int(r_init[k])
        g.r_splits_gen[k] = int(r_gen[k])
    if len(gens) > MAX_GEN:
        raise ValueError("at most %d generations" % MAX_GEN)
    g.num_generations = len(gens)
    for i, s in enumerate(gens):
        g.la_splits_gen[i] = int(s)
    return g


def stats_to_dict(s):
    return {
        "counts": [[int(s.counts[l][k]) for k in range(8)] for l in range(4)],
        "digest": int(s.digest),
        "leaf_evals": int(s.leaf_evals),
        "trapped_leaves": int(s.trapped_leaves),
        "gen_sizes": [int(s.gen_sizes[g]) for g in range(int(s.generations_run) + 1)],
        "generations_run": int(s.generations_run),
        "seconds": float(s.seconds),
        "kernel_launches": int(s.kernel_launches),
        "fp32_first": [int(x) for x in s.fp32_first],
        "cert_failures": int(s.cert_failures),
    }


_lib = None

EXPORTS = [
    "cc_create", "cc_destroy", "cc_status_str", "cc_last_error", "cc_tight_eval", "cc_tight_eval_device",
    "cc_last_launch_count", "cc_tight_prove", "cc_tight_prove_ex", "cc_tight_summary", "cc_interrupt", "cc_free",
    "cc_sb_eval", "cc_sb_eval_device", "cc_set_stage_timing", "cc_last_stage_times", "cc_sb_prove", "cc_sb_prove_ex",
    "cc_mlp_init", "cc_mlp_set_weights", "cc_mlp_get_weights", "cc_mlp_features", "cc_mlp_gradients",
    "cc_mlp_train_step", "cc_mlp_infer", "cc_tight_first", "cc_tight_cell_log", "cc_autotune_eval",
    "cc_tight_generation", "cc_set_checkpoint", "cc_tight_resume", "cc_last_eval_counts", "cc_set_eval_graph",
    "cc_eval_graph_stats", "cc_set_eval_certify", "cc_last_eval_cert", "cc_tight_refine", "cc_set_refine_order",
    "cc_sb_generation", "cc_tight_eval_device_static",
]

MLP_PARAMS = 5319
MLP_FEATURES = 10


def load_library(path=LIB_PATH):
    """Load the CUDA library (raises if it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise CudaError("CUDA library not built: %s (run __graft_entry__.build())" % path)
    lib = ctypes.CDLL(path)
    vp, sz = ctypes.c_void_p, ctypes.c_size_t
    lib.cc_create.argtypes = [ctypes.POINTER(vp), ctypes.c_int]
    lib.cc_destroy.argtypes = [vp]
    lib.cc_status_str.argtypes = [ctypes.c_int]
    lib.cc_status_str.restype = ctypes.c_char_p
    lib.cc_last_error.argtypes = [vp]
    lib.cc_last_error.restype = ctypes.c_char_p
    lib.cc_tight_eval.argtypes = [vp, vp, sz, vp]
    lib.cc_tight_eval_device.argtypes = [vp, vp, sz, vp, vp]
    lib.cc_tight_eval_device_static.argtypes = [vp, sz, vp, vp]
    lib.cc_last_launch_count.argtypes = [vp]
    lib.cc_last_launch_count.restype = ctypes.c_uint64
    missing = [name for name in EXPORTS if not hasattr(lib, name)]
    if missing:
        raise CudaError("library %s lacks %s" % (path, ", ".join(missing)))
    lib.cc_tight_prove.argtypes = [vp, ctypes.POINTER(CcTightBox), ctypes.POINTER(CcTightGrid), ctypes.POINTER(vp),
                                   ctypes.POINTER(sz), ctypes.POINTER(CcProveStats)]
    lib.cc_tight_prove_ex.argtypes = [vp, ctypes.POINTER(CcTightBox), ctypes.POINTER(CcTightGrid), ctypes.c_int,
                                      ctypes.POINTER(vp), ctypes.POINTER(sz), ctypes.POINTER(CcProveStats)]
    lib.cc_tight_summary.argtypes = [vp, vp, sz, ctypes.POINTER(CcTightSummary)]
    lib.cc_sb_eval.argtypes = [vp, vp, sz, vp]
    lib.cc_sb_eval_device.argtypes = [vp, vp, sz, vp, vp]
    lib.cc_interrupt.argtypes = [vp]
    lib.cc_mlp_init.argtypes = [vp, ctypes.c_uint64]
    lib.cc_mlp_set_weights.argtypes = [vp, vp]
    lib.cc_mlp_get_weights.argtypes = [vp, vp]
    lib.cc_mlp_features.argtypes = [vp, vp, sz, ctypes.c_float, vp]
    lib.cc_mlp_gradients.argtypes = [vp, vp, vp, sz, vp, ctypes.POINTER(ctypes.c_float)]
    lib.cc_mlp_train_step.argtypes = [vp, vp, vp, sz, ctypes.c_float, ctypes.POINTER(ctypes.c_float)]
    lib.cc_mlp_infer.argtypes = [vp, vp, sz, vp]
    lib.cc_tight_first.argtypes = [vp, vp, sz, ctypes.c_int, vp, vp]
    lib.cc_tight_cell_log.argtypes = [vp, vp, sz, ctypes.POINTER(sz), ctypes.POINTER(ctypes.c_int)]
    lib.cc_autotune_eval.argtypes = [vp, vp, sz, vp, ctypes.POINTER(CcTuneResult)]
    lib.cc_last_eval_counts.argtypes = [vp, vp]
    lib.cc_set_checkpoint.argtypes = [vp, ctypes.c_char_p]
    lib.cc_tight_resume.argtypes = [vp, ctypes.c_char_p, ctypes.POINTER(CcTightGrid), ctypes.c_int, ctypes.POINTER(vp),
                                    ctypes.POINTER(sz), ctypes.POINTER(CcProveStats)]
    lib.cc_tight_generation.argtypes = [vp, vp, sz, ctypes.c_int, vp, ctypes.c_uint64, ctypes.c_uint64, ctypes.c_int,
                                        ctypes.POINTER(vp), ctypes.POINTER(sz), ctypes.POINTER(CcProveStats)]
    lib.cc_sb_prove.argtypes = [vp, vp, ctypes.POINTER(CcSbGrid), ctypes.POINTER(vp), ctypes.POINTER(sz),
                                ctypes.POINTER(vp), ctypes.POINTER(CcSbProveStats)]
    lib.cc_sb_prove_ex.argtypes = [vp, vp, ctypes.POINTER(CcSbGrid), ctypes.c_int, ctypes.POINTER(vp),
                                   ctypes.POINTER(sz), ctypes.POINTER(vp), ctypes.POINTER(CcSbProveStats)]
    lib.cc_set_stage_timing.argtypes = [vp, ctypes.c_int]
    lib.cc_set_eval_graph.argtypes = [vp, ctypes.c_int]
    lib.cc_set_eval_certify.argtypes = [vp, ctypes.c_int]
    lib.cc_set_refine_order.argtypes = [vp, ctypes.c_int]
    lib.cc_last_eval_cert.argtypes = [vp, vp]
    lib.cc_eval_graph_stats.argtypes = [vp, ctypes.POINTER(ctypes.c_ulonglong), ctypes.POINTER(ctypes.c_ulonglong)]
    lib.cc_last_stage_times.argtypes = [vp, vp, ctypes.c_int, ctypes.POINTER(ctypes.c_int)]
    lib.cc_free.argtypes = [vp]
    if hasattr(lib, "cc_selftest_round"):
        lib.cc_selftest_round.argtypes = [vp, ctypes.c_int, ctypes.c_int, vp, vp, vp, sz]
        lib.cc_selftest_round_to_floats.argtypes = [vp, vp, sz, vp]
        lib.cc_selftest_subinterval.argtypes = [vp, vp, vp, vp, vp, sz, vp, vp]
        lib.cc_selftest_bisection_f32.argtypes = [vp, ctypes.c_int, vp, sz, vp, vp]
        lib.cc_selftest_bisection_width.argtypes = [vp, ctypes.c_int, vp, sz, vp, vp]
    _lib = lib
    return lib


def box_struct(b):
    s = CcTightBox()
    s.la.lb, s.la.ub = float(b["la"][0]), float(b["la"][1])
    for k in range(4):
        s.r[k].lb, s.r[k].ub = float(b["r"][k][0]), float(b["r"][k][1])
    return s


class Prover:
    """One CUDA device and stream; mirrors the reference's entry points."""

    def __init__(self, device=0):
        self.lib = load_library()
        h = ctypes.c_void_p()
        rc = self.lib.cc_create(ctypes.byref(h), int(device))
        if rc != 0:
            raise CudaError("cc_create(device=%d): %s" % (device, self.lib.cc_status_str(rc).decode()))
        self.h = h

    def close(self):
        if self.h:
            self.lib.cc_destroy(self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def _check(self, rc, what):
        if rc != 0:
            raise CudaError("%s: %s (%s)" % (what, self.lib.cc_status_str(rc).decode(),
                                             self.lib.cc_last_error(self.h).decode()))

    @property
    def last_launch_count(self):
        return int(self.lib.cc_last_launch_count(self.h))

    def tight_eval(self, boxes, out=None):
        """Verdict masks (TV_* bits) of host boxes (TIGHT_BOX records), into
        `out` (a uint32 host array, e.g. page-locked) if given."""
        boxes = np.ascontiguousarray(boxes, dtype=TIGHT_BOX)
        masks = np.zeros(len(boxes), dtype=np.uint32) if out is None else out
        if masks.dtype != np.uint32 or len(masks) != len(boxes) or not masks.flags["C_CONTIGUOUS"]:
            raise ValueError("out: a contiguous uint32 array of len(boxes)")
        self._check(self.lib.cc_tight_eval(self.h, boxes.ctypes.data, len(boxes), masks.ctypes.data), "cc_tight_eval")
        return masks

    def tight_eval_device(self, soa_ptr, n, masks_ptr, stream_ptr=None):
        """Device-resident variant: SoA (10 x n float64) in, uint32 masks out;
        asynchronous on `stream_ptr` (raw cudaStream_t) or the handle's stream."""
        self._check(self.lib.cc_tight_eval_device(self.h, ctypes.c_void_p(soa_ptr), n, ctypes.c_void_p(masks_ptr),
                                                  ctypes.c_void_p(stream_ptr) if stream_ptr else None),
                    "cc_tight_eval_device")

    def tight_eval_device_static(self, soa_ptr, n, masks_ptr, stream_ptr=None):
        """The allocation-free entry point (cc_tight_eval_device_static, no
        handle; at most 65,536 boxes per call, calls on one device must not
        overlap): same arguments as tight_eval_device."""
        self._check(self.lib.cc_tight_eval_device_static(ctypes.c_void_p(soa_ptr), n, ctypes.c_void_p(masks_ptr),
                                                         ctypes.c_void_p(stream_ptr) if stream_ptr else None),
                    "cc_tight_eval_device_static")

    def autotune_eval(self, soa_ptr, n, masks_ptr):
        """Tune the evaluation passes on a device sample (cc_autotune_eval);
        the choice stays in this handle.  Returns the report as a dict."""
        r = CcTuneResult()
        self._check(self.lib.cc_autotune_eval(self.h, ctypes.c_void_p(soa_ptr), n, ctypes.c_void_p(masks_ptr),
                                              ctypes.byref(r)), "cc_autotune_eval")
        return {k: {"min_blocks": r.min_blocks[i], "blocks_per_sm": r.blocks_per_sm[i],
                    "ms": float(r.ms[i]), "ms_default": float(r.ms_default[i])} for i, k in enumerate(TUNED_PASSES)}

    def set_eval_graph(self, enable=True):
        """Replay the evaluation's launch sequence as a CUDA graph while its
        arguments repeat (cc_set_eval_graph; on by default)."""
        self._check(self.lib.cc_set_eval_graph(self.h, int(bool(enable))), "cc_set_eval_graph")

    def eval_graph_stats(self):
        """(captures, replays) of the evaluation graph on this handle."""
        c, r = ctypes.c_ulonglong(), ctypes.c_ulonglong()
        self._check(self.lib.cc_eval_graph_stats(self.h, ctypes.byref(c), ctypes.byref(r)), "cc_eval_graph_stats")
        return int(c.value), int(r.value)

    def set_stage_timing(self, enable=True):
        """Record a CUDA event around each evaluation kernel (see stage_times)."""
        self._check(self.lib.cc_set_stage_timing(self.h, int(bool(enable))), "cc_set_stage_timing")

    def stage_times(self):
        """Milliseconds of the evaluation passes (EVAL_PASSES order) in the
        last timed evaluation (waits for it to finish)."""
        ms = np.zeros(len(EVAL_PASSES), dtype=np.float32)
        n = ctypes.c_int()
        self._check(self.lib.cc_last_stage_times(self.h, ms.ctypes.data, len(ms), ctypes.byref(n)),
                    "cc_last_stage_times")
        return [float(x) for x in ms[: n.value]]

    def set_eval_certify(self, enable=True):
        """FP64 certification of the evaluation's FP32 "true" verdicts (on by
        default); off is the uncertified FP32 form, for measurement only."""
        self._check(self.lib.cc_set_eval_certify(self.h, 1 if enable else 0), "cc_set_eval_certify")

    def eval_cert_counts(self):
        """Certification counts of the last evaluation batch: FP32 "true"
        verdicts certified per criterion group (r1, r1_r2, 2x2, leaf, three
        strips or emptiness), boxes whose certification failed (evaluated
        again in FP64), strip-width and gap-width results certified."""
        c = (ctypes.c_ulonglong * 8)()
        self._check(self.lib.cc_last_eval_cert(self.h, c), "cc_last_eval_cert")
        keys = ("r1", "r1_r2", "two_by_two", "leaf", "three_strips_or_empty", "failed", "cover", "gaps")
        return {k: int(v) for k, v in zip(keys, c)}

    def eval_counts(self):
        """Queue sizes of the last evaluation batch (cc_last_eval_counts):
        boxes left to the FP64 pass, strip-width and gap-width jobs."""
        c = (ctypes.c_ulonglong * 4)()
        self._check(self.lib.cc_last_eval_counts(self.h, c), "cc_last_eval_counts")
        return {"fp64_boxes": int(c[0]), "cover_jobs": int(c[1]), "gaps_jobs": int(c[2]), "overflow": int(c[3])}

    def sb_eval(self, boxes):
        """Size-bound verdict masks (CC_SV_* bits) of host boxes (SB_BOX records)."""
        boxes = np.ascontiguousarray(boxes, dtype=SB_BOX)
        masks = np.zeros(len(boxes), dtype=np.uint32)
        self._check(self.lib.cc_sb_eval(self.h, boxes.ctypes.data, len(boxes), masks.ctypes.data), "cc_sb_eval")
        return masks

    def sb_eval_device(self, soa_ptr, n, masks_ptr, stream_ptr=None):
        """Device-resident size-bound evaluation: SoA (14 x n float64) in."""
        self._check(self.lib.cc_sb_eval_device(self.h, ctypes.c_void_p(soa_ptr), n, ctypes.c_void_p(masks_ptr),
                                               ctypes.c_void_p(stream_ptr) if stream_ptr else None),
                    "cc_sb_eval_device")

    def tight_generation(self, parents, la_splits, r_splits, lo=0, hi=(1 << 64) - 1, learned=False):
        """One generation of the tight proof over the tasks [lo, hi)
        (cc_tight_generation): (criticals in task order, stats)."""
        parents = np.ascontiguousarray(parents, dtype=TIGHT_BOX)
        rs = (ctypes.c_int * 4)(*r_splits)
        out = ctypes.c_void_p()
        n = ctypes.c_size_t()
        st = CcProveStats()
        self._check(self.lib.cc_tight_generation(self.h, parents.ctypes.data if len(parents) else None, len(parents),
                                                 la_splits, rs, lo, hi, 4 if learned else 0, ctypes.byref(out),
                                                 ctypes.byref(n), ctypes.byref(st)), "cc_tight_generation")
        arr = np.zeros(n.value, dtype=TIGHT_BOX)
        if n.value:
            ctypes.memmove(arr.ctypes.data, out.value, n.value * TIGHT_BOX.itemsize)
        self.lib.cc_free(out)
        return arr, stats_to_dict(st)

    def set_checkpoint(self, path):
        """Write the tight proof's state after every generation to `path`
        (None: off)."""
        self._check(self.lib.cc_set_checkpoint(self.h, path.encode() if path else None), "cc_set_checkpoint")

    def tight_resume(self, path, grid=None, learned=False):
        """Continue a tight proof from a checkpoint: (criticals, stats)."""
        out = ctypes.c_void_p()
        n = ctypes.c_size_t()
        st = CcProveStats()
        self._check(self.lib.cc_tight_resume(self.h, path.encode(), ctypes.byref(grid) if grid is not None else None,
                                             4 if learned else 0, ctypes.byref(out), ctypes.byref(n), ctypes.byref(st)),
                    "cc_tight_resume")
        arr = np.zeros(n.value, dtype=TIGHT_BOX)
        if n.value:
            ctypes.memmove(arr.ctypes.data, out.value, n.value * TIGHT_BOX.itemsize)
        self.lib.cc_free(out)
        return arr, stats_to_dict(st)

    def tight_cell_log(self):
        """(cells, r4_splits) logged by the last proof run with log_cells=True."""
        n = ctypes.c_size_t()
        s4 = ctypes.c_int()
        self._check(self.lib.cc_tight_cell_log(self.h, None, 0, ctypes.byref(n), ctypes.byref(s4)), "cc_tight_cell_log")
        out = np.zeros(n.value, dtype=TIGHT_BOX)
        if n.value:
            self._check(self.lib.cc_tight_cell_log(self.h, out.ctypes.data, n.value, ctypes.byref(n), ctypes.byref(s4)),
                        "cc_tight_cell_log")
        return out, int(s4.value)

    def tight_find_critical_intervals(self, root, grid, plain=False, learned=False, log_cells=False):
        """The tight proof from `root` (a TIGHT_BOX record) with split counts
        `grid` (make_grid); returns (criticals, stats).  plain=True runs the
        plain form (every criterion re-evaluated in every cell); learned=True
        lets the trained network order the leaf criteria (CC_PROVE_LEARNED);
        log_cells=True keeps a sample of r3 cells for tight_cell_log()."""
        rs = box_struct(root)
        out = ctypes.c_void_p()
        n = ctypes.c_size_t()
        st = CcProveStats()
        flags = (1 if plain else 0) | (4 if learned else 0) | (8 if log_cells else 0)
        self._check(self.lib.cc_tight_prove_ex(self.h, ctypes.byref(rs), ctypes.byref(grid), flags,
                                               ctypes.byref(out), ctypes.byref(n), ctypes.byref(st)),
                    "cc_tight_prove_ex")
        arr = np.zeros(n.value, dtype=TIGHT_BOX)
        if n.value:
            ctypes.memmove(arr.ctypes.data, out.value, n.value * TIGHT_BOX.itemsize)
        self.lib.cc_free(out)
        return arr, stats_to_dict(st)

    def sb_find_critical_intervals(self, root, grid, plain=False, fp32=True):
        """The size-bound proof from `root` (an SB_BOX record) with split counts
        `grid` (make_sb_grid); returns (criticals, flags, stats).  Criticals
        are in the reference's final order (sorted and merged); flags bit 0 =
        kept because a criterion reached a trap site.  plain=True runs the
        plain form (one thread per leaf runs the whole cascade); fp32=False
        turns off the FP32 emptiness pre-filter.  All forms give the same
        criticals, flags and trace."""
        root = np.ascontiguousarray(np.asarray(root, dtype=SB_BOX).reshape(1))
        out = ctypes.c_void_p()
        flags = ctypes.c_void_p()
        n = ctypes.c_size_t()
        st = CcSbProveStats()
        opts = (1 if plain else 0) | (0 if fp32 else 2)
        self._check(self.lib.cc_sb_prove_ex(self.h, root.ctypes.data, ctypes.byref(grid), opts, ctypes.byref(out),
                                            ctypes.byref(n), ctypes.byref(flags), ctypes.byref(st)), "cc_sb_prove_ex")
        arr = np.zeros(n.value, dtype=SB_BOX)
        fl = np.zeros(n.value, dtype=np.uint32)
        if n.value:
            ctypes.memmove(arr.ctypes.data, out.value, n.value * SB_BOX.itemsize)
            ctypes.memmove(fl.ctypes.data, flags.value, n.value * 4)
        self.lib.cc_free(out)
        self.lib.cc_free(flags)
        d = sb_stats_to_dict(st)
        d["seconds"] = float(st.seconds)
        d["kernel_launches"] = int(st.kernel_launches)
        d["fp32_decided"] = int(st.fp32_decided)
        d["widening_samples"] = int(st.widening_samples)
        d["widening_mean"] = float(st.widening_mean)
        d["widening_max"] = float(st.widening_max)
        d["fp32_certified"] = int(st.fp32_certified)
        d["empty_anchors"] = int(st.empty_anchors)
        d["cert_failures"] = int(st.cert_failures)
        return arr, fl, d

    def sb_generation(self, parents, gen, la_splits, r_splits, lo=0, hi=(1 << 64) - 1, fp32=True):
        """One size-bound generation over the tasks [lo, hi)
        (cc_sb_generation): (criticals, flags, stats)."""
        parents = np.ascontiguousarray(np.asarray(parents, dtype=SB_BOX).reshape(-1))
        rs = (ctypes.c_int * 6)(*r_splits)
        out = ctypes.c_void_p()
        fl = ctypes.c_void_p()
        n = ctypes.c_size_t()
        st = CcSbProveStats()
        f = self.lib.cc_sb_generation
        f.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t, ctypes.c_int, ctypes.c_int, ctypes.c_void_p,
                      ctypes.c_uint64, ctypes.c_uint64, ctypes.c_int, ctypes.POINTER(ctypes.c_void_p),
                      ctypes.POINTER(ctypes.c_size_t), ctypes.POINTER(ctypes.c_void_p), ctypes.POINTER(CcSbProveStats)]
        self._check(f(self.h, parents.ctypes.data if len(parents) else None, len(parents), gen, la_splits, rs, lo, hi,
                      0 if fp32 else 2, ctypes.byref(out), ctypes.byref(n), ctypes.byref(fl), ctypes.byref(st)),
                    "cc_sb_generation")
        arr = np.zeros(n.value, dtype=SB_BOX)
        flags = np.zeros(n.value, dtype=np.uint32)
        if n.value:
            ctypes.memmove(arr.ctypes.data, out.value, n.value * SB_BOX.itemsize)
            ctypes.memmove(flags.ctypes.data, fl.value, n.value * 4)
        self.lib.cc_free(out)
        self.lib.cc_free(fl)
        d = sb_stats_to_dict(st)
        d["cert_failures"] = int(st.cert_failures)
        return arr, flags, d

    # ---- learned strategy ordering (device pointers are raw ints, e.g.
    # torch.Tensor.data_ptr())
    def mlp_init(self, seed=0):
        self._check(self.lib.cc_mlp_init(self.h, seed), "cc_mlp_init")

    def mlp_weights(self):
        w = np.zeros(MLP_PARAMS, dtype=np.float32)
        self._check(self.lib.cc_mlp_get_weights(self.h, w.ctypes.data), "cc_mlp_get_weights")
        return w

    def mlp_set_weights(self, w):
        w = np.ascontiguousarray(w, dtype=np.float32)
        assert w.size == MLP_PARAMS
        self._check(self.lib.cc_mlp_set_weights(self.h, w.ctypes.data), "cc_mlp_set_weights")

    def mlp_features(self, soa_ptr, n, feat_ptr, depth=0.0):
        self._check(self.lib.cc_mlp_features(self.h, ctypes.c_void_p(soa_ptr), n, depth, ctypes.c_void_p(feat_ptr)),
                    "cc_mlp_features")

    def mlp_gradients(self, feat_ptr, labels_ptr, n):
        g = np.zeros(MLP_PARAMS, dtype=np.float32)
        loss = ctypes.c_float()
        self._check(self.lib.cc_mlp_gradients(self.h, ctypes.c_void_p(feat_ptr), ctypes.c_void_p(labels_ptr), n,
                                              g.ctypes.data, ctypes.byref(loss)), "cc_mlp_gradients")
        return g, float(loss.value)

    def mlp_train_step(self, feat_ptr, labels_ptr, n, lr):
        loss = ctypes.c_float()
        self._check(self.lib.cc_mlp_train_step(self.h, ctypes.c_void_p(feat_ptr), ctypes.c_void_p(labels_ptr), n,
                                               lr, ctypes.byref(loss)), "cc_mlp_train_step")
        return float(loss.value)

    def mlp_infer(self, feat_ptr, n, logits_ptr):
        self._check(self.lib.cc_mlp_infer(self.h, ctypes.c_void_p(feat_ptr), n, ctypes.c_void_p(logits_ptr)),
                    "cc_mlp_infer")

    def tight_first(self, soa_ptr, n, outcome_ptr, evals_ptr=None, learned=False):
        """First-success evaluation (see cc_tight_first); device pointers."""
        self._check(self.lib.cc_tight_first(self.h, ctypes.c_void_p(soa_ptr), n, 1 if learned else 0,
                                            ctypes.c_void_p(outcome_ptr),
                                            ctypes.c_void_p(evals_ptr) if evals_ptr else None), "cc_tight_first")

    def tight_refine(self, boxes, max_depth, max_live=0, order="masks"):
        """Adaptive refinement of host boxes (cc_tight_refine): (criticals,
        flags, stats dict with per-depth live / decided counts, ms, queue
        occupancy and criterion steps).  order: "masks" (the certified
        evaluation of all criteria), "first_plain" or "first_learned"
        (cc_set_refine_order)."""
        self._check(self.lib.cc_set_refine_order(self.h, REFINE_ORDERS[order]), "cc_set_refine_order")
        boxes = np.ascontiguousarray(boxes, dtype=TIGHT_BOX)
        out = ctypes.c_void_p()
        fl = ctypes.c_void_p()
        n = ctypes.c_size_t()
        st = CcRefineStats()
        f = self.lib.cc_tight_refine
        f.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t, ctypes.c_int, ctypes.c_size_t,
                      ctypes.POINTER(ctypes.c_void_p), ctypes.POINTER(ctypes.c_void_p), ctypes.POINTER(ctypes.c_size_t),
                      ctypes.POINTER(CcRefineStats)]
        self._check(f(self.h, boxes.ctypes.data if len(boxes) else None, len(boxes), max_depth, max_live,
                      ctypes.byref(out), ctypes.byref(fl), ctypes.byref(n), ctypes.byref(st)), "cc_tight_refine")
        arr = np.zeros(n.value, dtype=TIGHT_BOX)
        flags = np.zeros(n.value, dtype=np.uint32)
        if n.value:
            ctypes.memmove(arr.ctypes.data, out.value, n.value * TIGHT_BOX.itemsize)
            ctypes.memmove(flags.ctypes.data, fl.value, n.value * 4)
        self.lib.cc_free(out)
        self.lib.cc_free(fl)
        d = int(st.depths_run)

        def per_depth(a):
            return [int(x) for x in a[:d]]
        return arr, flags, {"live": per_depth(st.live), "decided": per_depth(st.decided),
                            "ms": [float(x) for x in st.ms[:d]], "depths_run": d,
                            "stopped_at_cap": bool(st.stopped_at_cap), "seconds": float(st.seconds),
                            "kernel_launches": int(st.kernel_launches), "fp64_boxes": per_depth(st.fp64_boxes),
                            "cover_jobs": per_depth(st.cover_jobs), "gaps_jobs": per_depth(st.gaps_jobs),
                            "cert_jobs": per_depth(st.cert_jobs), "steps": per_depth(st.steps),
                            "warp_max_steps": per_depth(st.warp_max_steps), "cut": per_depth(st.cut),
                            "order": int(st.order)}

    def tight_summary(self, criticals):
        """Max_distances of a critical set (cc_tight_summary), as the raw
        cc_tight_summary_t structure."""
        crit = np.ascontiguousarray(criticals, dtype=TIGHT_BOX)
        out = CcTightSummary()
        self._check(self.lib.cc_tight_summary(self.h, crit.ctypes.data if len(crit) else None, len(crit),
                                              ctypes.byref(out)), "cc_tight_summary")
        return out

    def interrupt(self):
        self.lib.cc_interrupt(self.h)

    # diagnostics
    def selftest_round(self, op, up, a, b=None):
        a = np.ascontiguousarray(a, dtype=np.float64)
        bb = np.ascontiguousarray(b, dtype=np.float64) if b is not None else None
        out = np.empty_like(a)
        self._check(self.lib.cc_selftest_round(self.h, op, 1 if up else 0, a.ctypes.data,
                                               bb.ctypes.data if bb is not None else None, out.ctypes.data, len(a)),
                    "cc_selftest_round")
        return out

    def selftest_certify(self, group, boxes, call, record=False):
        """FP64 certification runs of criterion group `group` (0 r1, 1 r1_r2,
        2 2x2, 3 leaf r1_r2_r3) with call number call[i] per box (1-based;
        0 none; -1 all): bool array, the criterion held (record: in the
        record form the evaluation uses)."""
        boxes = np.ascontiguousarray(boxes, dtype=TIGHT_BOX)
        call = np.ascontiguousarray(call, dtype=np.int32)
        out = np.zeros(len(boxes), dtype=np.uint8)
        f = self.lib.cc_selftest_certify
        f.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t,
                      ctypes.c_void_p]
        self._check(f(self.h, group, boxes.ctypes.data, call.ctypes.data, len(boxes), out.ctypes.data),
                    "cc_selftest_certify")
        return ((out >> (1 if record else 0)) & 1).astype(bool)

    def selftest_round_to_floats(self, x):
        """(n, 4) floats per double: the FP32 enclosures' rounding down and up,
        then __double2float_rd / __double2float_ru."""
        x = np.ascontiguousarray(x, dtype=np.float64)
        out = np.empty((len(x), 4), dtype=np.float32)
        self._check(self.lib.cc_selftest_round_to_floats(self.h, x.ctypes.data, len(x), out.ctypes.data),
                    "cc_selftest_round_to_floats")
        return out

    def selftest_subinterval(self, lo, hi, idx, cnt):
        lo = np.ascontiguousarray(lo, dtype=np.float64)
        hi = np.ascontiguousarray(hi, dtype=np.float64)
        idx = np.ascontiguousarray(idx, dtype=np.int32)
        cnt = np.ascontiguousarray(cnt, dtype=np.int32)
        a = np.empty(2 * len(lo))
        b = np.empty(2 * len(lo))
        self._check(self.lib.cc_selftest_subinterval(self.h, lo.ctypes.data, hi.ctypes.data, idx.ctypes.data,
                                                     cnt.ctypes.data, len(lo), a.ctypes.data, b.ctypes.data),
                    "cc_selftest_subinterval")
        return a.reshape(-1, 2), b.reshape(-1, 2)

    def selftest_bisection_f32(self, which, args):
        """Bisection predicate decided by the FP32 enclosure over [lo, hi]
        (-1 undecided, 0, 1) and by the FP64 predicate at lo (0, 1; +2 on a
        trap), per row of 8 args (cc_selftest_bisection_f32; which 0 = cover
        strip, 1 = gaps; lo, hi in columns 6 and 7)."""
        args = np.ascontiguousarray(args, dtype=np.float64).reshape(-1, 8)
        f32 = np.empty(len(args), dtype=np.int8)
        f64 = np.empty(len(args), dtype=np.int8)
        self._check(self.lib.cc_selftest_bisection_f32(self.h, int(which), args.ctypes.data, len(args),
                                                       f32.ctypes.data, f64.ctypes.data), "cc_selftest_bisection_f32")
        return f32, f64

    def selftest_bisection_width(self, which, args):
        """The device's whole bisection per row (cc_selftest_bisection_width):
        (widths, trapped)."""
        args = np.ascontiguousarray(args, dtype=np.float64).reshape(-1, 8)
        out = np.empty(len(args))
        tr = np.empty(len(args), dtype=np.int8)
        self._check(self.lib.cc_selftest_bisection_width(self.h, int(which), args.ctypes.data, len(args),
                                                         out.ctypes.data, tr.ctypes.data), "cc_selftest_bisection_width")
        return out, tr
