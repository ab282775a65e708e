"""The allocation-free support filter (cmt_support_from_estimate_noalloc) against the
allocating entry point, called through the C ABI.

Callers that cannot allocate device memory (a host whose own memory pool has reserved the
GPU, or a latency-bound caller that cannot take a cudaMalloc's synchronisation) use the
allocation-free variant; it must give the same mask and the same masked estimate as
cmt_support_from_estimate with caller scratch, call after call, since every call reuses
one fixed device array.  This file is collected last.
"""
import ctypes

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def _ptr(t):
    return ctypes.c_void_p(t.data_ptr())


def _estimate(rng, M):
    est = rng.standard_normal((M,) * 3).astype(np.float32) * (rng.random((M,) * 3) > 0.4)
    est[rng.random((M,) * 3) > 0.8] = 1e-13  # values that straddle the 1e-12 threshold after smoothing
    return torch.from_numpy(est).cuda()


def test_noalloc_support_matches_allocating_entry_point():
    from cmtip_gb300 import _lib
    lib = _lib.load()
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    rng = np.random.default_rng(11)
    # two calls in a row per size: the second must not see anything left by the first
    for M in (81, 81, 37, 128):
        est = _estimate(rng, M)
        est_a, est_b = est.clone(), est.clone()
        sup_a = torch.empty_like(est)
        sup_b = torch.full_like(est, -7.0)
        scratch = torch.empty(2 * est.numel(), dtype=torch.float32, device="cuda")
        _lib.check(lib.cmt_support_from_estimate(_ptr(est_a), M, _ptr(sup_a), _ptr(scratch), 1, stream))
        _lib.check(lib.cmt_support_from_estimate_noalloc(_ptr(est_b), M, _ptr(sup_b), 1, stream))
        torch.cuda.synchronize()
        assert torch.equal(sup_a, sup_b)
        assert torch.equal(est_a, est_b)
        assert 0 < int(sup_b.sum()) < est.numel()


def test_noalloc_support_rejects_grids_beyond_its_scratch():
    from cmtip_gb300 import _lib
    lib = _lib.load()
    M = 129
    est = torch.zeros((M,) * 3, device="cuda")
    sup = torch.empty_like(est)
    rc = lib.cmt_support_from_estimate_noalloc(_ptr(est), M, _ptr(sup), 0,
                                               ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
    assert rc == _lib.CMT_ERR_ARG
    assert b"128" in lib.cmt_last_error()
