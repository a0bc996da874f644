"""bhr_trace_noalloc: the mixed-precision trace for callers that cannot allocate device memory
(render loops that must not stall on cudaMalloc, hosts whose pool owns all device memory, code
recording a CUDA graph). Its work memory is a static device array, so it is checked here
through the C ABI against the context-based entry point (bhr_trace, BHR_PREC_MIXED) on two
calls in a row (the second call reuses the array the first one left behind). Each ray's march
does not depend on the launch shape or on where the work memory lives, so the records must be
the same bytes; the parity report is kept to say where they differ if they ever do. This file
is collected last."""
import ctypes

import numpy as np
import pytest

import parity
from blackholerender_gb300 import PREC_MIXED, TERM_CONFIG, TERM_SHADER, Tracer, View, _abi, hits_numpy, make_view, workloads


def _noalloc(view, out_tensor, stream):
    return _abi.lib().bhr_trace_noalloc(ctypes.byref(view), ctypes.c_void_p(out_tensor.data_ptr()),
                                        ctypes.c_void_p(stream.cuda_stream))


def _same(a, b):
    if np.array_equal(a.view(np.uint8), b.view(np.uint8)):
        return
    rep = parity.compare(a, b, max_steps=10**9, band=0.0, edge_rel=0.0)
    differ = int(np.count_nonzero(np.any(a.view(np.uint8).reshape(-1, 64) != b.view(np.uint8).reshape(-1, 64), axis=1)))
    raise AssertionError(f"{differ} of {len(a)} records differ from bhr_trace's: {rep.as_dict()}")


@pytest.mark.gpu
@pytest.mark.parametrize("view", [
    workloads.c3_view(TERM_CONFIG, width=640, height=360),         # edge-on: band rays and FP64 hand-offs
    make_view(TERM_SHADER, width=480, height=270, fov_deg=60.0, preset=2, pose=(12.0, 1.3, 0.7)),
])
def test_noalloc_matches_trace_twice(view):
    import torch

    stream = torch.cuda.current_stream()
    with Tracer(0) as tr:
        (ref_out,) = tr.trace(view, precision=PREC_MIXED, stream=stream)
    torch.cuda.synchronize()
    ref = hits_numpy(ref_out.cpu())
    assert (ref["flags"] & 1).any()  # the FP64 path ran
    for _ in range(2):
        out = torch.full((view.rays * 64,), 0xAB, dtype=torch.uint8, device="cuda")  # stale bytes
        rc = _noalloc(view, out, stream)
        assert rc == 0, _abi.lib().bhr_last_error(None)
        torch.cuda.synchronize()
        _same(hits_numpy(out.cpu()), ref)


def test_noalloc_rejects_views_beyond_its_static_memory():
    v = make_view(TERM_CONFIG, width=1024, height=512)  # 524288 rays > 262144
    rc = _abi.lib().bhr_trace_noalloc(ctypes.byref(v), ctypes.c_void_p(16), ctypes.c_void_p(0))
    assert rc == _abi.ERR_INVALID_ARG
    msg = _abi.lib().bhr_last_error(None).decode()
    assert "262144" in msg and "524288" in msg
