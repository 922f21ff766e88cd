"""NT2's reductions (sum, asum1, asum2, norm2, mean, var, stdev, max, min, prod, all,
any, none) on the GPU, along dim 1, dim 2 and over the whole table.

The reference values are the FP64 evaluation of NT2's definitions
(modules/core/reduction/include/nt2/core/functions/expr/{asum1,asum2,norm2,mean,var,stdev}.hpp,
modules/boost/simd/reduction/functions/{sum,maximum,minimum,prod,all,any,none}.hpp):
  mean = rec(n) * sum,  var = f * sum((x - mean)^2) with f = 1/(n-1) (1/n for w = 1,
  1 when n <= 1),  stdev = sqrt(var),  norm2 = sqrt(sum(x^2)).
NT2's own FP32 folds combine partials in thread-arrival order, so FP32 results
are held to stated bounds against FP64 (eps = 2^-24):
  sum, asum1 (compensated):  4 eps |r| + 64 eps^2 n sum|x|
  asum2:                     6 eps r + 64 eps^2 n r       (each square rounds once)
  norm2:                     4 eps r + 32 eps^2 n r
  mean:                      (4 eps |S| + 64 eps^2 n sum|x|) / n + 2 eps |r|
  var, stdev (one pass):     64 eps (1 + kappa) r,   kappa = |mean| / stdev (+ 2 eps n^-1/2 for n < 64)
  prod:                      (n + 8) eps |r|
max, min, all, any and none are exact.
"""
import math

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

EPS = 2.0 ** -24
EPS64 = 2.0 ** -53


@pytest.fixture(params=["auto", "simt", "tma"], autouse=True)
def fold_path(request, cuda_lib):
    code = {"auto": 0, "simt": 1, "tma": 2}[request.param]
    assert cuda_lib.nt2cuda_set_fold_path(code) == 0
    yield request.param
    cuda_lib.nt2cuda_set_fold_path(0)


def to_dev(a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def host(t):
    torch.cuda.synchronize()
    return t.cpu().numpy()


def slices(A, rows, cols, dim):
    """FP64 view with one reduced slice per row of the result."""
    M = A.astype(np.float64).reshape(cols, rows)     # M[j] = column j of the column-major table
    if dim == 0:
        return M.reshape(1, rows * cols)
    return M if dim == 1 else M.T


def reference(op, S, w1=False):
    n = S.shape[1]
    if op == "sum":
        return S.sum(axis=1)
    if op == "asum1":
        return np.abs(S).sum(axis=1)
    if op == "asum2":
        return (S * S).sum(axis=1)
    if op == "norm2":
        return np.sqrt((S * S).sum(axis=1))
    if op == "mean":
        return S.sum(axis=1) / n if n else np.full(S.shape[0], np.nan)
    if op in ("var", "stdev"):
        if n == 0:
            v = np.zeros(S.shape[0])
        else:
            m = S.mean(axis=1, keepdims=True)
            f = 1.0 if n <= 1 else 1.0 / (n - (0 if w1 else 1))
            v = f * ((S - m) ** 2).sum(axis=1)
        return np.sqrt(v) if op == "stdev" else v
    if op == "max":
        return S.max(axis=1) if n else np.full(S.shape[0], -np.finfo(np.float32).max)
    if op == "min":
        return S.min(axis=1) if n else np.full(S.shape[0], np.finfo(np.float32).max)
    if op == "prod":
        return S.prod(axis=1)
    raise ValueError(op)


def bound(op, S, r):
    n = S.shape[1]
    ab = np.abs(S).sum(axis=1)
    if op in ("sum", "asum1"):
        return 4 * EPS * np.abs(r) + 64 * EPS * EPS * n * ab
    if op == "asum2":
        return 6 * EPS * r + 64 * EPS * EPS * n * r
    if op == "norm2":
        return 4 * EPS * r + 32 * EPS * EPS * n * r
    if op == "mean":
        return (4 * EPS * np.abs(S.sum(axis=1)) + 64 * EPS * EPS * n * ab) / max(n, 1) + 2 * EPS * np.abs(r)
    if op in ("var", "stdev"):
        sd = S.std(axis=1) if n else np.zeros(S.shape[0])
        kappa = np.abs(S.mean(axis=1)) / np.maximum(sd, 1e-300) if n else np.zeros(S.shape[0])
        rel = 64 * EPS * (1 + kappa) + (2 * EPS / math.sqrt(n) if 0 < n < 64 else 0)
        return rel * np.abs(r) + 1e-30
    if op == "prod":
        return (n + 8) * EPS * np.abs(r)
    return np.zeros_like(r)


SHAPES = [(1, 1), (5, 3), (31, 7), (33, 9), (1000, 17), (8192, 64), (4, 100000), (100000, 4), (257, 300),
          (1 << 17, 2)]
OPS = ["sum", "asum1", "asum2", "norm2", "mean", "var", "stdev", "max", "min"]


@pytest.mark.parametrize("shape", SHAPES)
@pytest.mark.parametrize("dim", [0, 1, 2])
def test_reductions_f32(gpu, shape, dim):
    rows, cols = shape
    rng = np.random.default_rng(rows * 7 + cols)
    A = (rng.standard_normal(rows * cols) * 3 + 1).astype(np.float32)
    Ad = to_dev(A)
    S = slices(A, rows, cols, dim)
    for op in OPS:
        got = host(gpu.reduce(op, Ad, rows, cols, dim)).astype(np.float64)
        r = reference(op, S)
        if op in ("max", "min"):
            assert np.array_equal(got, r), op
        else:
            err = np.abs(got - r)
            lim = bound(op, S, r)
            assert np.all(err <= lim), (op, int(np.argmax(err - lim)), float(np.max(err - lim)))


@pytest.mark.parametrize("mu", [0.0, 10.0, 1000.0])
@pytest.mark.parametrize("dim", [0, 1, 2])
@pytest.mark.parametrize("w1", [False, True])
def test_var_stdev_offset_data(gpu, mu, dim, w1):
    """var and stdev of data far from zero (kappa = |mean|/stdev up to 1000)."""
    rows, cols = 4096, 96
    rng = np.random.default_rng(int(mu) + 3)
    A = (rng.standard_normal(rows * cols) + mu).astype(np.float32)
    S = slices(A, rows, cols, dim)
    for op in ("var", "stdev"):
        got = host(gpu.reduce(op, to_dev(A), rows, cols, dim, var_by_n=w1)).astype(np.float64)
        r = reference(op, S, w1)
        assert np.all(np.abs(got - r) <= bound(op, S, r)), (op, float(np.max(np.abs(got - r) / r)))


@pytest.mark.parametrize("shape", [(1000, 7), (70000, 3), (3, 5000)])
@pytest.mark.parametrize("dim", [0, 1, 2])
def test_prod_f32(gpu, shape, dim):
    rows, cols = shape
    rng = np.random.default_rng(11)
    A = rng.uniform(0.999, 1.001, rows * cols).astype(np.float32)
    S = slices(A, rows, cols, dim)
    got = host(gpu.reduce("prod", to_dev(A), rows, cols, dim)).astype(np.float64)
    r = reference("prod", S)
    assert np.all(np.abs(got - r) <= bound("prod", S, r))


@pytest.mark.parametrize("shape", [(1, 1), (33, 9), (8192, 64), (100000, 4), (4, 100000)])
@pytest.mark.parametrize("dim", [0, 1, 2])
def test_logical_reductions(gpu, shape, dim):
    rows, cols = shape
    rng = np.random.default_rng(rows + cols)
    A = (rng.random(rows * cols) < 0.999).astype(np.float32)    # mostly nonzero
    A[rng.integers(0, A.size, 3)] = np.nan                       # NaN counts as nonzero
    S = slices(np.nan_to_num(A, nan=1.0), rows, cols, dim) != 0
    Ad = to_dev(A)
    assert np.array_equal(host(gpu.reduce("all", Ad, rows, cols, dim)), S.all(axis=1).astype(np.uint8))
    assert np.array_equal(host(gpu.reduce("any", Ad, rows, cols, dim)), S.any(axis=1).astype(np.uint8))
    assert np.array_equal(host(gpu.reduce("none", Ad, rows, cols, dim)), (~S.any(axis=1)).astype(np.uint8))
    Z = torch.zeros_like(Ad)
    assert not host(gpu.reduce("any", Z, rows, cols, dim)).any()
    assert host(gpu.reduce("none", Z, rows, cols, dim)).all()


def test_max_min_skip_nan(gpu):
    rows, cols = 1000, 8
    rng = np.random.default_rng(2)
    A = rng.standard_normal(rows * cols).astype(np.float32)
    A[::97] = np.nan
    S = slices(A, rows, cols, 1)
    assert np.array_equal(host(gpu.reduce("max", to_dev(A), rows, cols, 1)), np.nanmax(S, axis=1).astype(np.float32))
    assert np.array_equal(host(gpu.reduce("min", to_dev(A), rows, cols, 1)), np.nanmin(S, axis=1).astype(np.float32))


def test_empty_folds_give_neutral_values(gpu):
    """A fold of zero elements: NT2's neutral values, and mean = rec(0) * 0 = NaN."""
    A = torch.empty(0, device="cuda")
    big = np.finfo(np.float32).max
    expect = {"sum": 0.0, "asum1": 0.0, "asum2": 0.0, "norm2": 0.0, "var": 0.0, "stdev": 0.0, "max": -big,
              "min": big, "prod": 1.0}
    for op, v in expect.items():
        got = host(gpu.reduce(op, A, 0, 3, 1))
        assert np.array_equal(got, np.full(3, v, np.float32)), op
    assert np.all(np.isnan(host(gpu.reduce("mean", A, 0, 3, 1))))
    assert host(gpu.reduce("all", A, 0, 3, 1)).tolist() == [1, 1, 1]
    assert host(gpu.reduce("any", A, 0, 3, 1)).tolist() == [0, 0, 0]
    one = to_dev(np.array([5.0], np.float32))
    assert host(gpu.reduce("var", one, 1, 1, 1))[0] == 0.0     # n <= 1: f = 1, M2 = 0


def test_integer_valued_reductions_exact(gpu):
    """Integer-valued tables reduce exactly (modules/core/reduction/unit/table/sum.cpp:29-198)."""
    A = torch.arange(1, 13, dtype=torch.float32, device="cuda")   # 3x4 column-major
    assert host(gpu.reduce("sum", A, 3, 4, 1)).tolist() == [6, 15, 24, 33]
    assert host(gpu.reduce("sum", A, 3, 4, 2)).tolist() == [22, 26, 30]
    assert host(gpu.reduce("max", A, 3, 4, 1)).tolist() == [3, 6, 9, 12]
    assert host(gpu.reduce("min", A, 3, 4, 2)).tolist() == [1, 2, 3]
    assert host(gpu.reduce("prod", A, 3, 4, 1)).tolist() == [6, 120, 504, 1320]
    assert host(gpu.reduce("mean", A, 3, 4, 1)).tolist() == [2, 5, 8, 11]
    assert host(gpu.reduce("var", A, 3, 4, 1)).tolist() == [1, 1, 1, 1]
    assert host(gpu.reduce("asum1", -A, 3, 4, 0)).tolist() == [78]


@pytest.mark.parametrize("dim", [0, 1, 2])
def test_reductions_f64(gpu, dim):
    rows, cols = 3000, 40
    rng = np.random.default_rng(5)
    A = rng.standard_normal(rows * cols) * 2 + 3
    S = slices(A, rows, cols, dim)
    n = S.shape[1]
    for op in OPS + ["prod"]:
        X = A if op != "prod" else rng.uniform(0.999, 1.001, rows * cols)
        Sx = slices(X, rows, cols, dim)
        got = host(gpu.reduce(op, to_dev(X), rows, cols, dim))
        r = reference(op, Sx)
        tol = (math.log2(max(n, 2)) + 256) * EPS64 * (np.abs(Sx).sum(axis=1) if op != "prod" else n * np.abs(r))
        if op in ("asum2", "norm2"):
            tol = (math.log2(max(n, 2)) + 256) * EPS64 * (Sx * Sx).sum(axis=1)
        if op in ("var", "stdev"):
            tol = 1e-12 * np.abs(r)
        if op in ("max", "min"):
            assert np.array_equal(got, r), op
        else:
            assert np.all(np.abs(got - r) <= tol + 1e-300), op


def test_full_config_8192x4096_all_ops(gpu):
    """Every reduction of the 8192 x 4096 N(0,1) table along both dimensions, against FP64."""
    rows, cols = 8192, 4096
    Ad = torch.empty(rows * cols, device="cuda")
    gpu.fill_normal(Ad, 3)
    A = host(Ad)
    for dim in (1, 2):
        S = slices(A, rows, cols, dim)
        for op in OPS:
            got = host(gpu.reduce(op, Ad, rows, cols, dim)).astype(np.float64)
            r = reference(op, S)
            if op in ("max", "min"):
                assert np.array_equal(got, r), (op, dim)
            else:
                assert np.all(np.abs(got - r) <= bound(op, S, r)), (op, dim)
