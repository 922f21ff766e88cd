"""Bounded waits of the TMA folds: a block whose bulk copy never arrives gives
up, its column becomes NaN, the timeout is counted, and the arrival counters
of the stream's scratch are left at zero, so the next fold on the stream is
right.  (This module runs after the scan tests, which assert that none of
their own waits ran out.)"""
import ctypes as C

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

EPS = 2.0 ** -24


def _count(cuda_lib):
    c = C.c_ulonglong()
    assert cuda_lib.nt2cuda_wait_timeouts(C.byref(c)) == 0
    return c.value


def _check_colsums(got, A64):
    ref = A64.sum(axis=0)
    ab = np.abs(A64).sum(axis=0)
    assert np.all(np.abs(got.astype(np.float64) - ref) <= 4 * EPS * np.abs(ref) + 64 * EPS * EPS * A64.shape[0] * ab)


def test_fold_timeout_is_reported_and_counters_recover(gpu, cuda_lib):
    rows, cols = 3 * 65536 + 4, 3                      # every column is split into 4 units
    rng = np.random.default_rng(5)
    A = rng.standard_normal((cols, rows)).astype(np.float32)   # column-major: one row of A per column
    dA = torch.from_numpy(A.reshape(-1)).cuda()
    out = torch.full((cols,), 7.0, device="cuda")
    stream = torch.cuda.current_stream().cuda_stream
    c0 = _count(cuda_lib)
    st = cuda_lib.nt2cuda_selftest_fold_timeout(dA.data_ptr(), rows, cols, out.data_ptr(), stream)
    assert st == 5                                    # NT2CUDA_ERR_TIMEOUT
    assert _count(cuda_lib) == c0 + 1
    got = out.cpu().numpy()
    assert np.isnan(got[0])
    _check_colsums(got[1:], A[1:].T.astype(np.float64))
    # the next split fold on the same stream (TMA path) merges column 0 correctly
    assert cuda_lib.nt2cuda_set_fold_path(2) == 0
    try:
        out2 = torch.empty(cols, device="cuda")
        assert cuda_lib.nt2cuda_sum_inner_f32(dA.data_ptr(), rows, cols, out2.data_ptr(), 1, stream) == 0
        torch.cuda.synchronize()
        _check_colsums(out2.cpu().numpy(), A.T.astype(np.float64))
    finally:
        cuda_lib.nt2cuda_set_fold_path(0)
    assert _count(cuda_lib) == c0 + 1
