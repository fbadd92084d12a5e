"""In-tree build of the prover's CUDA library for sm_103a.

``libcirclecover_gb300.so`` (under ``circlecover_gb300/_build/``) exports the C
ABI of ``include/circlecover_gb300.h``.  The translation units are compiled in
parallel with nvcc and linked as a shared library; the prover's with
``-fmad=false`` (no implicit FMA contraction), the diagnostic one with nvcc's
default contraction on purpose.
"""
import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
OUT = os.path.join(PKG, "_build")
LIB = os.path.join(OUT, "libcirclecover_gb300.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-O2",
                 "--expt-relaxed-constexpr", "-I" + os.path.join(ROOT, "include")]
# --split-compile=0: the device code of a unit is compiled in parallel
# pieces (one process per core), the units themselves in parallel too
UNITS = [
    ("cc_prover.cu", ["-fmad=false", "-Xptxas", "-v", "--split-compile=0"]),
    ("cc_sb_kernels.cu", ["-fmad=false", "-Xptxas", "-v", "--split-compile=0"]),
    ("cc_sb_prove.cu", ["-fmad=false", "-Xptxas", "-v", "--split-compile=0"]),
    ("cc_mlp.cu", ["-fmad=false", "-Xptxas", "-v"]),
    ("cc_selftest_fmad.cu", []),
]


def nvcc():
    for c in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if c and (os.path.isabs(c) and os.path.exists(c) or not os.path.isabs(c)):
            return c
    return "nvcc"


def _deps():
    return [os.path.join(CSRC, f) for f in os.listdir(CSRC)] + [os.path.join(ROOT, "include", "circlecover_gb300.h")]


def _stale():
    if not os.path.exists(LIB):
        return True
    t = os.path.getmtime(LIB)
    return any(os.path.getmtime(d) > t for d in _deps()) or os.path.getmtime(__file__) > t


def _compile(unit):
    name, extra = unit
    src = os.path.join(CSRC, name)
    obj = os.path.join(OUT, name.replace(".cu", ".o"))
    cmd = [nvcc()] + COMMON + extra + ["-c", src, "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("nvcc failed for %s:\n%s\n%s" % (name, r.stdout, r.stderr))
    with open(obj + ".log", "w") as f:
        f.write(r.stdout + r.stderr)
    return obj


def build(force=False, verbose=False):
    """Compile (if stale) and return the path of the shared library."""
    os.makedirs(OUT, exist_ok=True)
    if not force and not _stale():
        return LIB
    with ThreadPoolExecutor(max_workers=len(UNITS)) as ex:
        objs = list(ex.map(_compile, UNITS))
    tmp = LIB + ".tmp%d" % os.getpid()
    cmd = [nvcc()] + ARCH + ["-shared", "-o", tmp] + objs + ["-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed:\n%s\n%s" % (r.stdout, r.stderr))
    os.replace(tmp, LIB)
    build_prover()
    if verbose:
        for name, _ in UNITS:
            log = os.path.join(OUT, name.replace(".cu", ".o.log"))
            sys.stdout.write(open(log).read())
    return LIB


PROVER = os.path.join(OUT, "circlecover_prover")


def build_prover():
    """The C++ host driver (drop-in for the reference's prover.cpp and its
    find_critical_intervals()) linked against the library."""
    host = os.path.join(PKG, "host")
    srcs = [os.path.join(host, f) for f in sorted(os.listdir(host)) if f.endswith(".cpp")]
    cxx = os.environ.get("CXX", "g++")
    tmp = PROVER + ".tmp%d" % os.getpid()
    cmd = [cxx, "-O2", "-std=c++17", "-I" + os.path.join(ROOT, "include")] + srcs + [
        "-L" + OUT, "-lcirclecover_gb300", "-Wl,-rpath,$ORIGIN", "-pthread", "-o", tmp]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("host driver build failed:\n%s\n%s" % (r.stdout, r.stderr))
    os.replace(tmp, PROVER)
    return PROVER


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
