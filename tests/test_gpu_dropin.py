"""GPU tier: the drop-in C++ drivers (circlecover_prover) and the interrupt
path of the proof.

* The binary's stdout equals the reference's output format built here from
  the CPU oracle's results: the 120-column case banners (output_case.hpp:
  35-54), the tight proof's two- and three-disk summaries
  (tight_rectangle.cu:508-533) and the size-bound proof's "Critical: " lines
  (rectangle_size_bound.cu:372-377), boxes and intervals in the reference's
  text format (tight_rectangle.cu:539-545, variables.hpp:112-118,
  interval.hpp:294-303: 19 significant digits, width 26).
* A first SIGINT stops the tight proof after the generation that is running
  (interrupt.cpp:30-46, tight_rectangle.cu:481-488) and the driver prints the
  summary of the last finished generation; cc_interrupt from another thread
  does the same through the C ABI.
"""
import ctypes
import os
import signal
import subprocess
import threading
import time

import numpy as np
import pytest

import circlecover_gb300 as cg
from circlecover_gb300 import workloads as W
from oracle import oracle as O

pytestmark = pytest.mark.gpu

WIDTH = 120
SB_GRID = "4:8,8,4,4,4,4:2:2,2,2,2,2,2:1"


def banner(msg):
    pre = (WIDTH - len(msg) - 2) // 2
    post = WIDTH - len(msg) - 2 - pre
    return "-" * pre + " " + msg + " " + "-" * post


def iv(lo, hi):
    return "[%26s, %26s]" % (format(lo, ".19g"), format(hi, ".19g"))


def tight_box_text(b):
    s = "λ = " + iv(*b["la"])
    for i in range(4):
        s += ", r²_%d = %s" % (i + 1, iv(*b["r"][i]))
    return s


def sb_box_text(b):
    s = "λ = " + iv(*b["la"])
    for i in range(6):
        s += ", r²_%d = %s" % (i + 1, iv(*b["r"][i]))
    return s


def summary_text(s, crit_boxes):
    """The reference's printing of Max_distances (tight_rectangle.cu:508-533)."""
    def box(c):
        return tight_box_text(np.frombuffer(bytes(c), dtype=W.TIGHT_BOX)[0])

    def ivs(x):
        return iv(x.lb, x.ub)

    out = []
    if s.have_range_2d:
        out.append("Two disks: Range for lambda that contains 2-disk critical intervals: %s; maximal distances "
                   "from theoretical values: " % ivs(s.la_range_2d))
        out.append("\tr_1^2: %s, r_2^2: %s, R_3 <= %s, h_1 >= %s, lambda / S_1 <= %s" % (
            ivs(s.dist_r1_2d), ivs(s.dist_r2_2d), format(s.ub_R3_2d, "g"), format(s.lb_h1_2d, "g"),
            format(s.ub_la_by_S1, "g")))
        out += ["\tDominating criticals for r_1: ", "\t\t" + box(s.dist_r1_2d_criticals[0]),
                "\t\t" + box(s.dist_r1_2d_criticals[1]), "\tDominating criticals for r_2: ",
                "\t\t" + box(s.dist_r2_2d_criticals[0]), "\t\t" + box(s.dist_r2_2d_criticals[1])]
    if s.have_range_3d:
        out.append("Three disks: Range for lambda that contains 3-disk critical intervals: %s; maximal distances "
                   "from theoretical values: " % ivs(s.la_range_3d))
        out.append("\tr_1^2: %s, r_2^2: %s, r_3^2: %s, R_4 <= %s" % (
            ivs(s.dist_r1_3d), ivs(s.dist_r2_3d), ivs(s.dist_r3_3d), format(s.ub_R4_3d, "g")))
        out.append("\tS_1: %s, h_2: %s, S_3: %s, pocket width <= %s" % (ivs(s.S1), ivs(s.h2), ivs(s.S3),
                                                                         format(s.pocket_width_3d, "g")))
        out += ["\tDominating criticals for r_1: ", "\t\t" + box(s.dist_r1_3d_criticals[0]),
                "\t\t" + box(s.dist_r1_3d_criticals[1]), "\tDominating criticals for r_2: ",
                "\t\t" + box(s.dist_r2_3d_criticals[0]), "\t\t" + box(s.dist_r2_3d_criticals[1]),
                "\tDominating criticals for r_3: ", "\t\t" + box(s.dist_r3_3d_criticals[0]),
                "\t\t" + box(s.dist_r3_3d_criticals[1])]
    return out


def port_summary(port, boxes):
    out = cg.CcTightSummary()
    f = port.lib.ccport_tight_summary
    f.argtypes = [ctypes.c_void_p, ctypes.c_size_t, ctypes.POINTER(cg.CcTightSummary)]
    boxes = np.ascontiguousarray(boxes, dtype=W.TIGHT_BOX)
    f(boxes.ctypes.data if len(boxes) else None, len(boxes), ctypes.byref(out))
    return out


class CkptHeader(ctypes.Structure):
    """Head of the tight proof's checkpoint file (the boxes follow it)."""
    _fields_ = [("magic", ctypes.c_char * 8), ("version", ctypes.c_uint32), ("next_gen", ctypes.c_int32),
                ("flags", ctypes.c_int32), ("pad", ctypes.c_int32), ("grid", cg.CcTightGrid),
                ("counts", (ctypes.c_uint64 * 8) * 4), ("digest", ctypes.c_uint64), ("leaf_evals", ctypes.c_uint64),
                ("trapped", ctypes.c_uint64), ("gen_sizes", ctypes.c_uint64 * (cg.MAX_GEN + 1)),
                ("n_parents", ctypes.c_uint64)]


def read_checkpoint(path):
    data = open(path, "rb").read()
    hd = CkptHeader.from_buffer_copy(data[:ctypes.sizeof(CkptHeader)])
    boxes = np.frombuffer(data[ctypes.sizeof(CkptHeader):], dtype=W.TIGHT_BOX)
    assert len(boxes) == hd.n_parents
    return hd, boxes


def expected_stdout(port, tight_crit, sb_crit, sb_flags):
    lines = [banner("Critical intervals for rectangles (tight)")]
    if len(tight_crit):
        lines += summary_text(port_summary(port, tight_crit), tight_crit)
    lines.append("-" * WIDTH)
    lines.append(banner("Critical intervals for rectangles with small disks"))
    for b, f in zip(sb_crit, sb_flags):
        lines.append(("Trapped: " if f else "Critical: ") + sb_box_text(b))
    lines.append("-" * WIDTH)
    return "\n".join(lines) + "\n"


def test_dropin_driver_stdout_and_sigint(port, tmp_path):
    from circlecover_gb300 import _build
    exe = _build.build_prover()
    ckpt = str(tmp_path / "tight.ckpt")
    env = dict(os.environ, CC_TIGHT_CHECKPOINT=ckpt, CC_SB_GRID=SB_GRID)
    env.pop("CC_TIGHT_GRID", None)
    env.pop("CC_TIGHT_LAMBDA_MAX", None)
    proc = subprocess.Popen([exe], stdout=subprocess.PIPE, stderr=subprocess.PIPE, env=env, text=True)
    # the full tight proof, reference schedule: its first refinement
    # generation takes seconds; interrupt once the initial pass is on disk
    t0 = time.time()
    while not os.path.exists(ckpt) and proc.poll() is None and time.time() - t0 < 300:
        time.sleep(0.01)
    assert proc.poll() is None, proc.stderr.read()[-2000:]
    proc.send_signal(signal.SIGINT)
    out, err = proc.communicate(timeout=600)
    assert proc.returncode == 0, err[-2000:]
    hd, tight_crit = read_checkpoint(ckpt)
    assert hd.next_gen >= 2  # the interrupt came after the initial pass
    assert hd.next_gen <= 1 + hd.grid.num_generations
    sgrid = [int(x) for x in SB_GRID.replace(":", ",").split(",")]
    sc, sf, _ = port.sb_prove(W.sb_root(1.0, 2.5), cg.make_sb_grid(sgrid[0], sgrid[1:7], sgrid[7], sgrid[8:14],
                                                                   sgrid[14]), threads=16)
    assert len(sc) > 0
    want = expected_stdout(port, tight_crit, sc, sf)
    assert out == want, "\n".join(l for l in difflib_lines(want, out))


def difflib_lines(a, b):
    import difflib
    return list(difflib.unified_diff(a.splitlines(), b.splitlines(), lineterm=""))[:40]


def test_dropin_driver_prints_the_summary_of_a_small_grid(port):
    """No interrupt: a narrow lambda range and small splits leave criticals,
    whose summary and the size-bound lines match the oracle's."""
    from circlecover_gb300 import _build
    exe = _build.build_prover()
    env = dict(os.environ, CC_TIGHT_LAMBDA_MAX="1.02", CC_TIGHT_GRID="8:16,32,32,32:1:16,16,16,16",
               CC_SB_GRID=SB_GRID)
    env.pop("CC_TIGHT_CHECKPOINT", None)
    r = subprocess.run([exe], capture_output=True, text=True, env=env, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    root = W.tight_root(1.0, 1.02)
    tc, _ = port.tight_prove(root, O.make_grid(8, (16, 32, 32, 32), gens=(1,), r_gen=(16, 16, 16, 16)), threads=16)
    assert len(tc) > 0
    sgrid = [int(x) for x in SB_GRID.replace(":", ",").split(",")]
    sc, sf, _ = port.sb_prove(W.sb_root(1.0, 2.5), cg.make_sb_grid(sgrid[0], sgrid[1:7], sgrid[7], sgrid[8:14],
                                                                   sgrid[14]), threads=16)
    want = expected_stdout(port, tc, sc, sf)
    assert r.stdout == want, "\n".join(difflib_lines(want, r.stdout))


def test_interrupt_stops_after_the_running_generation(tmp_path):
    """cc_interrupt from another thread, once the initial pass is done: the
    proof returns CC_ERR_INTERRUPTED with the criticals of the generation
    that was running when it came, equal to a proof that ends there."""
    ckpt = str(tmp_path / "int.ckpt")
    root = W.tight_root()
    grid = cg.make_grid(256, (128, 128, 128, 128), (1, 2, 2, 2, 2, 1, 2, 1, 2, 1, 2), (128, 128, 128, 64))
    p = cg.Prover(0)
    try:
        p.set_checkpoint(ckpt)
        lib = p.lib
        rs = cg.box_struct(root)
        out = ctypes.c_void_p()
        n = ctypes.c_size_t()
        st = cg.CcProveStats()
        res = {}

        def run():
            res["rc"] = lib.cc_tight_prove_ex(p.h, ctypes.byref(rs), ctypes.byref(grid), 0, ctypes.byref(out),
                                              ctypes.byref(n), ctypes.byref(st))

        th = threading.Thread(target=run)
        th.start()
        t0 = time.time()
        while not os.path.exists(ckpt) and th.is_alive() and time.time() - t0 < 300:
            time.sleep(0.005)
        p.interrupt()
        th.join(timeout=600)
        assert not th.is_alive()
        assert res["rc"] == 5  # CC_ERR_INTERRUPTED
        got = np.zeros(n.value, dtype=W.TIGHT_BOX)
        if n.value:
            ctypes.memmove(got.ctypes.data, out.value, n.value * W.TIGHT_BOX.itemsize)
        lib.cc_free(out)
        gens_run = int(st.generations_run)
        assert gens_run >= 1  # the interrupt came after the initial pass
        # the same proof stopped by its schedule after that generation
        p.set_checkpoint(None)
        short = cg.make_grid(256, (128, 128, 128, 128), (1, 2, 2, 2, 2, 1, 2, 1, 2, 1, 2)[:gens_run],
                             (128, 128, 128, 64))
        want, wst = p.tight_find_critical_intervals(root, short)
        assert np.array_equal(got.view(np.uint64), want.view(np.uint64))
        assert [int(st.gen_sizes[g]) for g in range(gens_run + 1)] == wst["gen_sizes"]
        assert int(st.digest) == wst["digest"]
    finally:
        p.close()
