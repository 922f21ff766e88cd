"""inner_fold / outer_fold reductions on the GPU.

NT2's own FP32 folds combine partials in thread-arrival order
(modules/arch/openmp/include/nt2/sdk/openmp/spawner/fold.hpp:49-66), so they
are not reproducible bit for bit; the oracle for FP32 folds is the FP64
(compensated) sum, and the stated bounds are
    compensated: |gpu - fp64| <= 4 eps |fp64| + 64 eps^2 n sum|x|
    plain:       |gpu - fp64| <= (log2(n) + 256) eps sum|x|
with eps = 2^-24 (FP32 unit roundoff).  The NT2-order FP32 sum's own error
is reported beside them.  Integer-valued tables must sum exactly.
"""
import math

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

EPS = 2.0 ** -24


def to_dev(a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


@pytest.fixture(params=["auto", "simt", "tma"], autouse=True)
def fold_path(request, cuda_lib):
    """Every fold test runs on each kernel family (nt2cuda_set_fold_path)."""
    code = {"auto": 0, "simt": 1, "tma": 2}[request.param]
    assert cuda_lib.nt2cuda_set_fold_path(code) == 0
    yield request.param
    cuda_lib.nt2cuda_set_fold_path(0)


def host(t):
    torch.cuda.synchronize()
    return t.cpu().numpy()


def bound(comp, n, ref, abs_sum):
    if comp:
        return 4 * EPS * abs(ref) + 64 * EPS * EPS * n * abs_sum
    return (math.log2(max(n, 2)) + 256) * EPS * abs_sum


@pytest.mark.parametrize("n", [0, 1, 5, 31, 32, 33, 1000, 16384, 16385, 100003, 1 << 22])
@pytest.mark.parametrize("comp", [True, False])
def test_globalsum_f32(gpu, oracle, n, comp):
    x = np.random.default_rng(n).standard_normal(n).astype(np.float32)
    got = float(host(gpu.globalsum(to_dev(x), compensated=comp))[0])
    ref, ab = oracle.sum_fp64(x)
    assert abs(got - ref) <= bound(comp, n, ref, ab) + (0 if n else 0), (n, got, ref)


@pytest.mark.parametrize("n", [1, 7, 16384 * 3 + 5, 1 << 22])
@pytest.mark.parametrize("comp", [True, False])
def test_dot_f32(gpu, oracle, n, comp):
    rng = np.random.default_rng(n + 1)
    x = rng.standard_normal(n).astype(np.float32)
    y = rng.standard_normal(n).astype(np.float32)
    got = float(host(gpu.dot(to_dev(x), to_dev(y), compensated=comp))[0])
    ref, ab = oracle.dot_fp64(x, y)
    # the float product rounding adds eps*sum|xy| to either form
    assert abs(got - ref) <= bound(comp, n, ref, ab) + EPS * ab, (n, got, ref)


def test_dot_full_size_reproducible(gpu, oracle):
    """sdot at 2^26: within the compensated bound, and bitwise identical run to run."""
    n = 1 << 26
    xd = torch.empty(n, dtype=torch.float32, device="cuda")
    yd = torch.empty(n, dtype=torch.float32, device="cuda")
    gpu.fill_normal(xd, 1)
    gpu.fill_normal(yd, 2)
    a = host(gpu.dot(xd, yd))[0]
    b = host(gpu.dot(xd, yd))[0]
    assert a.view(np.uint32) == b.view(np.uint32)
    x, y = host(xd), host(yd)
    ref, ab = oracle.dot_fp64(x, y)
    assert abs(float(a) - ref) <= bound(True, n, ref, ab) + EPS * ab
    plain = float(host(gpu.dot(xd, yd, compensated=False))[0])
    nt2_order = oracle.load().nt2o_dot_nt2_f(x, y, n, 8)
    # report: compensated error should not exceed the plain error by more than rounding noise
    assert abs(float(a) - ref) <= abs(plain - ref) + 2 * EPS * abs(ref) + EPS * ab
    assert math.isfinite(nt2_order)


@pytest.mark.parametrize("rows,cols", [(1, 1), (5, 3), (31, 7), (32, 5), (33, 9), (1000, 17), (8192, 64),
                                       (16384 * 2 + 3, 3), (4, 100000), (257, 1)])
@pytest.mark.parametrize("comp", [True, False])
def test_sum_inner_f32(gpu, oracle, rows, cols, comp):
    A = np.random.default_rng(rows * 31 + cols).standard_normal(rows * cols).astype(np.float32)
    got = host(gpu.sum_colmajor(to_dev(A), rows, cols, 1, compensated=comp))
    _, r64, a64 = oracle.inner_fold(A, rows, cols)
    for j in range(cols):
        assert abs(float(got[j]) - r64[j]) <= bound(comp, rows, r64[j], a64[j]), (j, got[j], r64[j])


@pytest.mark.parametrize("rows,cols", [(1, 1), (5, 3), (31, 7), (128, 256), (129, 257), (1000, 17),
                                       (8192, 64), (3, 5000), (4, 100000), (100000, 4)])
@pytest.mark.parametrize("comp", [True, False])
def test_sum_outer_f32(gpu, oracle, rows, cols, comp):
    A = np.random.default_rng(rows * 17 + cols).standard_normal(rows * cols).astype(np.float32)
    got = host(gpu.sum_colmajor(to_dev(A), rows, cols, 2, compensated=comp))
    r32, r64, a64 = oracle.outer_fold(A, rows, cols)
    err = np.abs(got.astype(np.float64) - r64)
    lim = np.array([bound(comp, cols, r64[i], a64[i]) for i in range(rows)])
    assert np.all(err <= lim), (np.argmax(err - lim),)


def test_fold_full_config_8192x4096(gpu, oracle):
    """inner_fold column sums and outer_fold row sums of an 8192x4096 N(0,1) table."""
    rows, cols = 8192, 4096
    Ad = torch.empty(rows * cols, dtype=torch.float32, device="cuda")
    gpu.fill_normal(Ad, 3)
    A = host(Ad)
    cs = host(gpu.sum_colmajor(Ad, rows, cols, 1))
    rs = host(gpu.sum_colmajor(Ad, rows, cols, 2))
    c32, c64, ca = oracle.inner_fold(A, rows, cols)
    r32, r64, ra = oracle.outer_fold(A, rows, cols)
    assert np.all(np.abs(cs - c64) <= 4 * EPS * np.abs(c64) + 64 * EPS * EPS * rows * ca)
    assert np.all(np.abs(rs - r64) <= 4 * EPS * np.abs(r64) + 64 * EPS * EPS * cols * ra)
    # the compensated GPU sums are at least as close to FP64 as NT2's own FP32 orders, in aggregate
    assert np.abs(cs - c64).sum() <= np.abs(c32 - c64).sum()
    assert np.abs(rs - r64).sum() <= np.abs(r32 - r64).sum()
    # reproducible
    assert np.array_equal(host(gpu.sum_colmajor(Ad, rows, cols, 2)).view(np.uint32), rs.view(np.uint32))


@pytest.mark.parametrize("comp", [True, False])
def test_sums_that_overflow_read_inf(gpu, comp):
    """A float sum that overflows is inf, as NT2's plain float sum gives, on the
    compensated path too (its compensation turns NaN once the sum is infinite);
    a NaN term still gives NaN."""
    x = np.ones(100000, np.float32)
    x[5000:5004] = np.float32(3.0e38)
    assert np.isposinf(float(host(gpu.globalsum(to_dev(x), compensated=comp))[0]))
    A = np.ones((4, 3000), np.float32)     # column-major 3000 x 4
    A[1, 10:14] = np.float32(3.0e38)
    A[2, 7] = np.nan
    flat = A.reshape(-1)
    cs = host(gpu.sum_colmajor(to_dev(flat), 3000, 4, 1, compensated=comp))
    assert cs[0] == 3000 and np.isposinf(cs[1]) and np.isnan(cs[2]) and cs[3] == 3000
    M = np.ones((3000, 4), np.float32)     # column-major 4 x 3000: row sums along dim 2
    M[10:14, 1] = np.float32(3.0e38)
    rs = host(gpu.sum_colmajor(to_dev(M.reshape(-1)), 4, 3000, 2, compensated=comp))
    assert rs[0] == 3000 and np.isposinf(rs[1]) and rs[2] == 3000


def test_integer_valued_sums_exact(gpu):
    # modules/core/reduction/unit/table/globalsum.cpp:22-30 and sum.cpp:29-198
    a = torch.arange(1, 10, dtype=torch.float32, device="cuda")
    assert float(host(gpu.globalsum(a))[0]) == 45.0
    a[8] = 0
    assert float(host(gpu.globalsum(a))[0]) == 36.0
    A = torch.arange(1, 13, dtype=torch.float32, device="cuda")   # 3x4 column-major
    assert host(gpu.sum_colmajor(A, 3, 4, 1)).tolist() == [6, 15, 24, 33]
    assert host(gpu.sum_colmajor(A, 3, 4, 2)).tolist() == [22, 26, 30]
    big = torch.ones(1 << 24, dtype=torch.float32, device="cuda")
    assert float(host(gpu.globalsum(big, compensated=False))[0]) == float(1 << 24)
    empty = torch.empty(0, dtype=torch.float32, device="cuda")
    assert float(host(gpu.globalsum(empty))[0]) == 0.0


@pytest.mark.parametrize("n", [1, 1000, 1 << 20])
def test_f64_folds(gpu, oracle, n):
    x = np.random.default_rng(n).standard_normal(n)
    got = float(host(gpu.globalsum(to_dev(x)))[0])
    ref, ab = oracle.sum_fp64(x)
    assert abs(got - ref) <= (math.log2(max(n, 2)) + 256) * 2.0 ** -53 * ab
    A = np.random.default_rng(2).standard_normal(256 * 300)
    cs = host(gpu.sum_colmajor(to_dev(A), 256, 300, 1))
    rs = host(gpu.sum_colmajor(to_dev(A), 256, 300, 2))
    M = A.reshape(300, 256)
    assert np.allclose(cs, M.sum(axis=1), rtol=0, atol=1e-12)
    assert np.allclose(rs, M.sum(axis=0), rtol=0, atol=1e-12)


def test_fold_after_fold_shares_scratch_safely(gpu, oracle):
    """A row-sum fold with split columns, then a column-sum fold with split rows on the same
    stream: the second fold's arrival counters must not see the first fold's partials."""
    rng = np.random.default_rng(12)
    B = rng.standard_normal(2048 * 3000).astype(np.float32)
    host(gpu.sum_colmajor(to_dev(B), 2048, 3000, 2))          # outer fold, partials in scratch
    rows, cols = 40000, 100                                  # inner fold: 3 segments per column
    A = rng.standard_normal(rows * cols).astype(np.float32)
    got = host(gpu.sum_colmajor(to_dev(A), rows, cols, 1))
    _, r64, a64 = oracle.inner_fold(A, rows, cols)
    for j in range(cols):
        assert abs(float(got[j]) - r64[j]) <= bound(True, rows, r64[j], a64[j]), j
