"""GPU test of cc_tight_eval_device_static, the allocation-free entry point.

It serves callers that cannot allocate device memory while they run: a host
framework that owns all device memory and hands out its own buffers, a
latency-critical loop in which cudaMalloc's implicit synchronisation would
stall the device, a process that reserves everything at start-up.  Instead of
handle-owned queues it works in a fixed array compiled into the library.

The test calls it through the C ABI twice in a row on different batches --
the second call reuses the array the first one filled -- and checks both
outputs bit for bit against cc_tight_eval_device (the entry point with
handle-owned buffers) and against the CPU oracle's masks.  After a warm-up
call it checks that a call leaves the device's free memory unchanged, and it
runs one call on a non-default stream.  The device buffers below are the
caller's (made with torch); the entry point itself allocates nothing.

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


def _device_entry_masks(boxes):
    """Masks from the existing device entry point (handle-owned scratch)."""
    import torch
    import circlecover_gb300 as cg
    soa, masks = _device_batch(boxes)
    torch.cuda.synchronize()
    with cg.Prover(0) as p:
        p.tight_eval_device(soa.data_ptr(), len(boxes), masks.data_ptr())
        torch.cuda.synchronize()
        return masks.cpu().numpy().view(np.uint32)


def _oracle_masks(boxes):
    from oracle import oracle as O
    O.ensure_built()
    return O.Port().tight_eval(boxes, threads=16)


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
        assert np.array_equal(got, _device_entry_masks(boxes))
        assert np.array_equal(got, _oracle_masks(boxes))


def test_static_entry_point_allocates_nothing_and_runs_on_a_stream():
    import torch
    lib = _lib()
    boxes = W.tight_microbench(30000, seed=74)
    soa, masks = _device_batch(boxes)
    warm_soa, warm_masks = _device_batch(boxes[:1])
    # the caller's stream, made (like every buffer above) before the part of
    # the program that must not allocate
    stream = torch.cuda.Stream()
    assert stream.cuda_stream != 0
    torch.cuda.synchronize()
    # warm-up on that stream: the one-time set-up and the loading of the kernels
    assert lib.cc_tight_eval_device_static(warm_soa.data_ptr(), 1, warm_masks.data_ptr(),
                                           ctypes.c_void_p(stream.cuda_stream)) == 0
    stream.synchronize()
    free_before = torch.cuda.mem_get_info()[0]
    rc = lib.cc_tight_eval_device_static(soa.data_ptr(), len(boxes), masks.data_ptr(),
                                         ctypes.c_void_p(stream.cuda_stream))
    assert rc == 0
    stream.synchronize()
    free_after = torch.cuda.mem_get_info()[0]
    assert free_after == free_before, (free_before, free_after)
    assert np.array_equal(masks.cpu().numpy().view(np.uint32), _oracle_masks(boxes))


def test_static_entry_point_rejects_oversized_batch():
    import torch
    lib = _lib()
    boxes = W.tight_microbench(8, seed=73)
    soa, masks = _device_batch(boxes)
    torch.cuda.synchronize()
    assert lib.cc_tight_eval_device_static(soa.data_ptr(), MAX_BOXES + 1, masks.data_ptr(), None) == TOO_LARGE
    assert lib.cc_tight_eval_device_static(None, 0, None, None) == 0
