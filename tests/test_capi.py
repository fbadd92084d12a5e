"""CPU tier: the C-ABI library builds for sm_103a, loads without a GPU and
exports every function include/circlecover_gb300.h declares; the Python
mirror fails loudly instead of falling back to the CPU."""
import ctypes
import os
import re

import pytest

from conftest import ROOT

HEADER = os.path.join(ROOT, "include", "circlecover_gb300.h")


def declared_functions():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    names = re.findall(r"^\s*(?:const\s+)?[a-z_0-9]+\s*\**\s+(cc_[a-z_0-9]+)\s*\(", text, flags=re.M)
    return sorted(set(names))


def test_header_declares_the_entry_points():
    names = declared_functions()
    for n in ["cc_create", "cc_destroy", "cc_tight_eval", "cc_tight_eval_device", "cc_tight_prove", "cc_tight_summary"]:
        assert n in names


def test_library_exports_every_declared_function(lib_path):
    lib = ctypes.CDLL(lib_path)
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, missing


def test_library_is_built_for_sm103a_only(lib_path):
    log = open(os.path.join(os.path.dirname(lib_path), "cc_prover.o.log")).read()
    assert "sm_103a" in log
    assert "spill" in log


def test_create_without_gpu_fails_loudly(lib_path):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    import circlecover_gb300 as cg
    with pytest.raises(cg.CudaError):
        cg.Prover(0)


def test_status_strings(lib_path):
    lib = ctypes.CDLL(lib_path)
    lib.cc_status_str.restype = ctypes.c_char_p
    assert lib.cc_status_str(0) == b"ok"
    assert b"overflow" in lib.cc_status_str(3)


def test_null_arguments_are_rejected(lib_path):
    lib = ctypes.CDLL(lib_path)
    assert lib.cc_create(None, 0) == 2
    assert lib.cc_tight_eval(None, None, 0, None) == 2
    assert lib.cc_tight_prove(None, None, None, None, None, None) == 2
    assert lib.cc_set_eval_graph(None, 1) == 2
    assert lib.cc_eval_graph_stats(None, None, None) == 2
    assert lib.cc_selftest_round_to_floats(None, None, ctypes.c_size_t(0), None) == 2
    assert lib.cc_sb_prove(None, None, None, None, None, None, None) == 2
    assert lib.cc_autotune_eval(None, None, ctypes.c_size_t(0), None, None) == 2
