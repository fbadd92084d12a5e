"""ORACLE / TEST INFRASTRUCTURE ONLY.

Builds the CPU oracle libraries:

* ``oracle/_build/libccport.so`` and ``libccport_count.so`` -- the CPU port
  (the prover's criteria headers compiled for the host with the exact
  directed-rounding layer); built everywhere, including the GPU machine.
* ``oracle/_ref/libccref.so`` -- the reference's own criteria sources compiled
  for the host (``oracle/ref/Makefile``); built only where the reference
  sources are present.

Run ``python oracle/build.py [--ref PATH]``.  The reference's ``Prover/``
directory is taken from ``--ref``, else from the environment variable
``CC_REFERENCE_PROVER``, else from a checkout of the reference beside this
repository (``<repo>/../reference/Prover``); without one, only the port is
built.
"""
import argparse
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
BUILD = os.path.join(HERE, "_build")
REF_OUT = os.path.join(HERE, "_ref")

PORT_FLAGS = [
    "-std=c++17", "-O2", "-fPIC", "-shared", "-pthread",
    "-frounding-math", "-ffp-contract=off", "-fno-fast-math",
]


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("command failed: %s\n%s%s" % (" ".join(cmd), r.stdout, r.stderr))


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _port_deps():
    deps = [os.path.join(HERE, "port", "port.cpp"), os.path.join(HERE, "tight_driver.hpp"),
            os.path.join(HERE, "shim", "cc_rounding.h"), os.path.join(ROOT, "include", "circlecover_gb300.h"),
            os.path.join(HERE, "sb_driver.hpp")]
    csrc = os.path.join(ROOT, "circlecover_gb300", "csrc")
    deps += [os.path.join(csrc, f) for f in os.listdir(csrc) if f.endswith(".cuh")]
    return deps


def build_port(force=False):
    os.makedirs(BUILD, exist_ok=True)
    src = os.path.join(HERE, "port", "port.cpp")
    cxx = os.environ.get("CXX", "g++")
    outs = []
    for name, extra in (("libccport.so", []), ("libccport_count.so", ["-DCC_PORT_COUNT"])):
        out = os.path.join(BUILD, name)
        if force or _stale(out, _port_deps()):
            tmp = out + ".tmp%d" % os.getpid()
            _run([cxx] + PORT_FLAGS + extra + ["-o", tmp, src])
            os.replace(tmp, out)
        outs.append(out)
    return outs


def reference_dir():
    """The reference's Prover/ directory when the reference is checked out
    beside this repository, else None."""
    d = os.path.normpath(os.path.join(ROOT, os.pardir, "reference", "Prover"))
    return d if os.path.isdir(d) else None


def build_ref(ref=None, force=False):
    """Build the reference criteria library; returns its path or None if the
    reference sources are not available here."""
    ref = ref or os.environ.get("CC_REFERENCE_PROVER") or reference_dir()
    if not ref or not os.path.isdir(ref):
        return None
    cmd = ["make", "-s", "-C", os.path.join(HERE, "ref"), "REF=" + ref, "-j%d" % (os.cpu_count() or 4)]
    if force:
        _run(["make", "-s", "-C", os.path.join(HERE, "ref"), "REF=" + ref, "clean"])
    _run(cmd)
    return os.path.join(REF_OUT, "libccref.so")


def build_ref_fenv(ref=None):
    """The fesetround variant of the reference criteria library
    (oracle/_ref/libccref_fe.so), for the CPU baseline's timing; None where
    the reference sources are not available."""
    ref = ref or os.environ.get("CC_REFERENCE_PROVER") or reference_dir()
    if not ref or not os.path.isdir(ref):
        return None
    _run(["make", "-s", "-C", os.path.join(HERE, "ref"), "REF=" + ref, "-j%d" % (os.cpu_count() or 4), "fenv"])
    return os.path.join(REF_OUT, "libccref_fe.so")


if __name__ == "__main__":
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", default=None)
    ap.add_argument("--force", action="store_true")
    a = ap.parse_args()
    print(build_port(a.force))
    print(build_ref(a.ref, a.force))
    sys.exit(0)
