"""CPU tier: the bench's reference arm keeps the JSON-line contract (one
line from rank 0, the CPU implementation timed on a bounded sample), alone
and under torchrun with two ranks."""
import json
import os
import socket
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _json_lines(out):
    return [json.loads(l) for l in out.splitlines() if l.startswith("{")]


def _check_line(line):
    assert line["impl"] == "reference"
    assert line["value"] > 0 and line["unit"] == "boxes/s" and line["higher_is_better"] is True
    assert line["cpu_baseline"]["kind"] in ("reference", "port") and line["cpu_baseline"]["cores"] >= 1
    assert line["cpu_baseline"]["value"] == line["value"]
    assert line["e2e"] == {"value": line["value"], "unit": "boxes/s", "h2d_bytes_per_step": 0,
                           "d2h_bytes_per_step": 0}


def test_reference_arm_prints_one_line():
    r = subprocess.run([sys.executable, "bench.py", "--impl", "reference", "--steps", "1", "--warmup", "0",
                        "--cpu-sample", "32768"], cwd=ROOT, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = _json_lines(r.stdout)
    assert len(lines) == 1, r.stdout[-2000:]
    _check_line(lines[0])
    assert lines[0]["config"]["boxes_per_step"] == 32768


def test_reference_arm_under_two_ranks():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    r = subprocess.run([sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
                        "--master-addr", "127.0.0.1", "--master-port", str(port), "bench.py", "--impl", "reference",
                        "--gpus", "2", "--steps", "1", "--warmup", "0", "--cpu-sample", "16384"],
                       cwd=ROOT, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = _json_lines(r.stdout)
    assert len(lines) == 1, r.stdout[-2000:]
    _check_line(lines[0])
    assert lines[0]["n_gpus"] == 2


def test_roofline_inputs_are_committed():
    """The bench's roofline reads per-box ncu counts of every evaluation pass
    from the committed profile summary; each pass has all five counts, and
    the pass rooflines and the HBM view come out finite from them."""
    sys.path.insert(0, ROOT)
    import bench
    import circlecover_gb300 as cg
    per_box = bench.profile_per_box()
    metrics = ("warp_inst", "thread_inst", "fp64_inst", "fp32_inst", "dram_bytes")
    for name in cg.EVAL_PASSES:
        assert all(m in per_box.get(name, {}) for m in metrics), name
    pk = {"fp64": 0.53e12, "issue": 1.2e12}
    stage_ms = [10.0, 0.5, 5.0, 2.5, 13.0, 0.01]
    passes = bench.pass_rooflines(stage_ms, 1 << 24, pk, per_box)
    assert passes["k_eval_cert"]["bound"] == "fp64" and 0 < passes["k_eval_cert"]["fp64_useful_frac"] < 2
    assert passes["k_eval_f32"]["bound"] == "issue" and 0 < passes["k_eval_f32"]["issue_frac"] < 2
    hv = bench.hbm_view(passes["k_eval_cert"]["traffic_bytes"], 13.0)
    assert hv["unit"] == "GB/s" and hv["achieved"] > 0
