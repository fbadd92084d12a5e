"""GPU test of cc_tight_eval_device_static, the allocation-free entry point.

It serves callers that cannot allocate device memory while they run (a host
framework that owns all device memory, latency-critical loops, processes that
reserve everything at start-up): instead of handle-owned queues it works in a
fixed array compiled into the library.  The test calls it through the C ABI
twice in a row on different batches -- the second call reuses the array the
first one filled -- and checks both outputs bit for bit against
cc_tight_eval_device, the entry point with handle-owned buffers.  The device
buffers below are the caller's (made with torch); the entry point itself
allocates nothing.

Kept in a file of its own that pytest collects last.
"""
import ctypes

import numpy as np
import pytest

from circlecover_gb300 import workloads as W

pytestmark = pytest.mark.gpu

MAX_BOXES = 65536
TOO_LARGE = 8


def _lib():
    from circlecover_gb300 import _build
    lib = ctypes.CDLL(_build.build())
    lib.cc_tight_eval_device_static.argtypes = [ctypes.c_void_p, ctypes.c_size_t, ctypes.c_void_p, ctypes.c_void_p]
    lib.cc_tight_eval_device_static.restype = ctypes.c_int
    return lib


def _device_batch(boxes):
    import torch
    soa = torch.from_numpy(W.to_soa(boxes)).cuda()
    masks = torch.full((len(boxes),), -1, dtype=torch.int32, device="cuda")
    return soa, masks


def _reference_masks(boxes):
    """Masks from the existing device entry point (handle-owned scratch)."""
    import torch
    import circlecover_gb300 as cg
    soa, masks = _device_batch(boxes)
    torch.cuda.synchronize()
    with cg.Prover(0) as p:
        p.tight_eval_device(soa.data_ptr(), len(boxes), masks.data_ptr())
        torch.cuda.synchronize()
        return masks.cpu().numpy().view(np.uint32)


def test_static_entry_point_matches_device_entry_point_twice():
    import torch
    lib = _lib()
    # two different batches, the second one smaller: the array keeps the
    # first call's queues, which the second call must not pick up
    batches = [W.tight_microbench(MAX_BOXES, seed=71), W.tight_near_critical(40000, seed=72)]
    outs = []
    for boxes in batches:
        soa, masks = _device_batch(boxes)
        torch.cuda.synchronize()
        rc = lib.cc_tight_eval_device_static(soa.data_ptr(), len(boxes), masks.data_ptr(), None)
        assert rc == 0
        torch.cuda.synchronize()
        outs.append(masks.cpu().numpy().view(np.uint32).copy())
    for boxes, got in zip(batches, outs):
        want = _reference_masks(boxes)
        assert np.array_equal(got, want)


def test_static_entry_point_rejects_oversized_batch():
    import torch
    lib = _lib()
    boxes = W.tight_microbench(8, seed=73)
    soa, masks = _device_batch(boxes)
    torch.cuda.synchronize()
    assert lib.cc_tight_eval_device_static(soa.data_ptr(), MAX_BOXES + 1, masks.data_ptr(), None) == TOO_LARGE
    assert lib.cc_tight_eval_device_static(None, 0, None, None) == 0
