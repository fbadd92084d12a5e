"""ORACLE / TEST INFRASTRUCTURE ONLY -- the checker, never the product.

ctypes bindings to the two CPU oracles:

* ``Ref``  -- the reference's own criteria (oracle/_ref/libccref.so, built from
  the reference sources where they exist) plus the restated driver loops;
* ``Port`` -- the prover's criteria headers compiled for the host
  (oracle/_build/libccport.so), pinned to ``Ref`` by the CPU tests.

Only ``tests/``, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline
leg use this module.
"""
import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)

TIGHT_BOX = np.dtype([("la", "<f8", (2,)), ("r", "<f8", (4, 2))])
SB_BOX = np.dtype([("la", "<f8", (2,)), ("r", "<f8", (6, 2))])
assert TIGHT_BOX.itemsize == 80 and SB_BOX.itemsize == 112


class CcIv(ctypes.Structure):
    _fields_ = [("lb", ctypes.c_double), ("ub", ctypes.c_double)]


class CcTightBox(ctypes.Structure):
    _fields_ = [("la", CcIv), ("r", CcIv * 4)]


MAX_GEN = 32


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


def make_grid(la_init, r_init, gens=(), r_gen=(128, 128, 128, 64)):
    g = CcTightGrid()
    g.la_splits_init = la_init
    for k in range(4):
        g.r_splits_init[k] = r_init[k]
        g.r_splits_gen[k] = r_gen[k]
    g.num_generations = len(gens)
    for i, s in enumerate(gens):
        g.la_splits_gen[i] = s
    return g


def stats_to_dict(s):
    return {
        "counts": [[int(s.counts[l][k]) for k in range(8)] for l in range(4)],
        "digest": int(s.digest),
        "leaf_evals": int(s.leaf_evals),
        "trapped_leaves": int(s.trapped_leaves),
        "gen_sizes": [int(s.gen_sizes[g]) for g in range(int(s.generations_run) + 1)],
        "generations_run": int(s.generations_run),
    }


def box_to_struct(b):
    s = CcTightBox()
    s.la.lb, s.la.ub = float(b[0][0]), float(b[0][1])
    for k in range(4):
        s.r[k].lb, s.r[k].ub = float(b[1][k][0]), float(b[1][k][1])
    return s


class _Lib:
    prefix = None

    def __init__(self, path):
        self.path = path
        self.lib = ctypes.CDLL(path)
        p = self.prefix
        f = getattr(self.lib, p + "_tight_eval")
        f.argtypes = [ctypes.c_void_p, ctypes.c_size_t, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int]
        f.restype = ctypes.c_int
        f = getattr(self.lib, p + "_tight_prove")
        f.argtypes = [ctypes.POINTER(CcTightBox), ctypes.POINTER(CcTightGrid), ctypes.c_int,
                      ctypes.POINTER(ctypes.c_void_p), ctypes.POINTER(ctypes.c_size_t), ctypes.POINTER(CcProveStats)]
        f.restype = ctypes.c_int
        getattr(self.lib, p + "_free").argtypes = [ctypes.c_void_p]

    def tight_eval(self, boxes, threads=1, count_ops=False):
        boxes = np.ascontiguousarray(boxes, dtype=TIGHT_BOX)
        n = len(boxes)
        masks = np.zeros(n, dtype=np.uint32)
        ops = np.zeros(n, dtype=np.uint64) if count_ops else None
        getattr(self.lib, self.prefix + "_tight_eval")(
            boxes.ctypes.data, n, masks.ctypes.data, ops.ctypes.data if ops is not None else None, threads)
        return (masks, ops) if count_ops else masks

    def sb_eval(self, boxes, threads=1, count_ops=False):
        boxes = np.ascontiguousarray(boxes, dtype=SB_BOX)
        n = len(boxes)
        masks = np.zeros(n, dtype=np.uint32)
        ops = np.zeros(n, dtype=np.uint64) if count_ops else None
        f = getattr(self.lib, self.prefix + "_sb_eval")
        f.argtypes = [ctypes.c_void_p, ctypes.c_size_t, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int]
        f(boxes.ctypes.data, n, masks.ctypes.data, ops.ctypes.data if ops is not None else None, threads)
        return (masks, ops) if count_ops else masks

    def tight_prove(self, root, grid, threads=1):
        out = ctypes.c_void_p()
        n = ctypes.c_size_t()
        st = CcProveStats()
        rs = box_to_struct(root)
        rc = getattr(self.lib, self.prefix + "_tight_prove")(ctypes.byref(rs), ctypes.byref(grid), threads,
                                                           ctypes.byref(out), ctypes.byref(n), ctypes.byref(st))
        if rc != 0:
            raise RuntimeError("prove failed %d" % rc)
        arr = np.zeros(n.value, dtype=TIGHT_BOX)
        if n.value:
            ctypes.memmove(arr.ctypes.data, out.value, n.value * TIGHT_BOX.itemsize)
        getattr(self.lib, self.prefix + "_free")(out)
        return arr, stats_to_dict(st)


    def sb_generation(self, parents, gen, la_splits, r_splits, lo=0, hi=(1 << 64) - 1, threads=1):
        """One size-bound generation over the tasks [lo, hi) on the host,
        merged as generation `gen`: (criticals, flags, stats dict)."""
        from circlecover_gb300 import CcSbProveStats, sb_stats_to_dict
        parents = np.ascontiguousarray(np.asarray(parents, dtype=SB_BOX).reshape(-1))
        rs = (ctypes.c_int * 6)(*r_splits)
        out = ctypes.c_void_p()
        flags = ctypes.c_void_p()
        n = ctypes.c_size_t()
        st = CcSbProveStats()
        f = getattr(self.lib, self.prefix + "_sb_generation")
        f.argtypes = [ctypes.c_void_p, ctypes.c_size_t, ctypes.c_int, ctypes.c_int, ctypes.c_void_p, ctypes.c_uint64,
                      ctypes.c_uint64, ctypes.c_int, ctypes.POINTER(ctypes.c_void_p), ctypes.POINTER(ctypes.c_void_p),
                      ctypes.POINTER(ctypes.c_size_t), ctypes.c_void_p]
        f(parents.ctypes.data if len(parents) else None, len(parents), gen, la_splits, rs, lo, hi, threads,
          ctypes.byref(out), ctypes.byref(flags), ctypes.byref(n), ctypes.addressof(st))
        arr = np.zeros(n.value, dtype=SB_BOX)
        fl = np.zeros(n.value, dtype=np.uint32)
        if n.value:
            ctypes.memmove(arr.ctypes.data, out.value, n.value * SB_BOX.itemsize)
            ctypes.memmove(fl.ctypes.data, flags.value, n.value * 4)
        getattr(self.lib, self.prefix + "_free")(out)
        getattr(self.lib, self.prefix + "_free")(flags)
        return arr, fl, sb_stats_to_dict(st)

    def sb_prove(self, root, grid, threads=1):
        """The size-bound proof on the host: (criticals SB_BOX array, flags, stats dict)."""
        from circlecover_gb300 import CcSbProveStats, sb_stats_to_dict
        root = np.ascontiguousarray(np.asarray(root, dtype=SB_BOX).reshape(1))
        out = ctypes.c_void_p()
        flags = ctypes.c_void_p()
        n = ctypes.c_size_t()
        st = CcSbProveStats()
        f = getattr(self.lib, self.prefix + "_sb_prove")
        f.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int, ctypes.POINTER(ctypes.c_void_p),
                      ctypes.POINTER(ctypes.c_void_p), ctypes.POINTER(ctypes.c_size_t), ctypes.c_void_p]
        rc = f(root.ctypes.data, ctypes.addressof(grid), threads, ctypes.byref(out), ctypes.byref(flags), ctypes.byref(n),
               ctypes.addressof(st))
        if rc != 0:
            raise RuntimeError("sb prove failed %d" % rc)
        arr = np.zeros(n.value, dtype=SB_BOX)
        fl = np.zeros(n.value, dtype=np.uint32)
        if n.value:
            ctypes.memmove(arr.ctypes.data, out.value, n.value * SB_BOX.itemsize)
            ctypes.memmove(fl.ctypes.data, flags.value, n.value * 4)
        getattr(self.lib, self.prefix + "_free")(out)
        getattr(self.lib, self.prefix + "_free")(flags)
        return arr, fl, sb_stats_to_dict(st)


class _Generation:
    def tight_generation(self, parents, la_splits, r_splits, lo=0, hi=(1 << 64) - 1, threads=4):
        """One generation over the tasks [lo, hi) on the CPU: (criticals in
        task order, stats)."""
        parents = np.ascontiguousarray(parents, dtype=TIGHT_BOX)
        rs = (ctypes.c_int * 4)(*r_splits)
        out = ctypes.c_void_p()
        n = ctypes.c_size_t()
        st = CcProveStats()
        f = getattr(self.lib, self.prefix + "_tight_generation")
        f.argtypes = [ctypes.c_void_p, ctypes.c_size_t, ctypes.c_int, ctypes.c_void_p, ctypes.c_uint64,
                      ctypes.c_uint64, ctypes.c_int, ctypes.POINTER(ctypes.c_void_p), ctypes.POINTER(ctypes.c_size_t),
                      ctypes.POINTER(CcProveStats)]
        f(parents.ctypes.data if len(parents) else None, len(parents), la_splits, rs, lo, hi, threads,
          ctypes.byref(out), ctypes.byref(n), ctypes.byref(st))
        arr = np.zeros(n.value, dtype=TIGHT_BOX)
        if n.value:
            ctypes.memmove(arr.ctypes.data, out.value, n.value * TIGHT_BOX.itemsize)
        getattr(self.lib, self.prefix + "_free")(out)
        return arr, stats_to_dict(st)


class Ref(_Generation, _Lib):
    """The reference's own criteria code, built for the host."""
    prefix = "ccref"

    def __init__(self, path=None):
        super().__init__(path or os.path.join(HERE, "_ref", "libccref.so"))
        self.lib.ccref_tight_critical_ratio.argtypes = [ctypes.c_double, ctypes.c_double, ctypes.POINTER(ctypes.c_double)]
        self.lib.ccref_tight_critical_ratio.restype = ctypes.c_double


class Port(_Generation, _Lib):
    """The prover's criteria compiled for the host (restatement)."""
    prefix = "ccport"

    def __init__(self, path=None, count=False):
        name = "libccport_count.so" if count else "libccport.so"
        super().__init__(path or os.path.join(HERE, "_build", name))
        self.lib.ccport_round.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p,
                                          ctypes.c_void_p, ctypes.c_size_t]
        self.lib.ccport_subinterval.argtypes = [ctypes.c_double, ctypes.c_double, ctypes.c_int, ctypes.c_int,
                                                ctypes.POINTER(ctypes.c_double)]

    def tight_eval_passes(self, boxes):
        """Per-box operation counts of the three evaluation passes (main,
        strip-width bisection, gap-width bisection); counting build only."""
        boxes = np.ascontiguousarray(boxes, dtype=TIGHT_BOX)
        ops3 = np.zeros((len(boxes), 3), dtype=np.uint64)
        f = self.lib.ccport_tight_eval_passes
        f.argtypes = [ctypes.c_void_p, ctypes.c_size_t, ctypes.c_void_p]
        f(boxes.ctypes.data, len(boxes), ops3.ctypes.data)
        return ops3

    def round(self, op, up, a, b=None, exact_fenv=False):
        a = np.ascontiguousarray(a, dtype=np.float64)
        bb = np.ascontiguousarray(b, dtype=np.float64) if b is not None else None
        out = np.empty_like(a)
        self.lib.ccport_round(op, 1 if up else 0, 1 if exact_fenv else 0, a.ctypes.data,
                              bb.ctypes.data if bb is not None else None, out.ctypes.data, len(a))
        return out

    def subinterval(self, lo, hi, i, n):
        out = (ctypes.c_double * 2)()
        self.lib.ccport_subinterval(lo, hi, i, n, out)
        return out[0], out[1]


def ref_available():
    return os.path.exists(os.path.join(HERE, "_ref", "libccref.so"))


def ensure_built():
    """Build the port (and the reference library where its sources exist)."""
    import importlib.util
    spec = importlib.util.spec_from_file_location("cc_oracle_build", os.path.join(HERE, "build.py"))
    m = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(m)
    m.build_port()
    m.build_ref()
