"""Cumulative functions (cumsum, cumprod, cummax, cummin) on the GPU along dim 1 and dim 2.

NT2 folds `summary = bop(summary, x)` in index order
(modules/core/swar/include/nt2/core/functions/details/scan_step.hpp:32-44); its
OpenMP spawner rescans blocks from the earlier blocks' summaries, so FP32
cumsum is not the sequential sum either.  The reference here is the FP64
running value, with the bounds (eps = 2^-24, cabs_i = running sum of |x|):
  cumsum, compensated:  4 eps |r_i| + 64 eps^2 n cabs_i
  cumsum, plain:        (tiles + 64) eps cabs_i        (tiles = ceil(n / 8192))
  cumprod:              (i + 16) eps |r_i|
cummax and cummin are exact (NaNs are skipped).  Every result must also be
bitwise identical from run to run.
"""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

EPS = 2.0 ** -24


def to_dev(a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def host(t):
    torch.cuda.synchronize()
    return t.cpu().numpy()


def lines(A, rows, cols, dim):
    """FP64 array whose rows are the scanned lines, and the map back to the flat layout."""
    M = A.astype(np.float64).reshape(cols, rows)
    return M if dim == 1 else M.T


def back(L, rows, cols, dim):
    return (L if dim == 1 else L.T).reshape(-1)


def check_cumsum(got, A, rows, cols, dim, comp):
    L = lines(A, rows, cols, dim)
    r = back(np.cumsum(L, axis=1), rows, cols, dim)
    cabs = back(np.cumsum(np.abs(L), axis=1), rows, cols, dim)
    n = L.shape[1]
    if comp:
        lim = 4 * EPS * np.abs(r) + 64 * EPS * EPS * n * cabs
    else:
        lim = ((n + 8191) // 8192 + 64) * EPS * cabs
    err = np.abs(got.astype(np.float64) - r)
    assert np.all(err <= lim), (int(np.argmax(err - lim)), float(np.max(err - lim)))


SHAPES = [(1, 1), (7, 3), (64, 5), (65, 5), (1000, 17), (8192, 3), (8193, 2), (100003, 2), (3, 1000)]


@pytest.mark.parametrize("shape", SHAPES)
@pytest.mark.parametrize("dim", [1, 2])
@pytest.mark.parametrize("comp", [True, False])
def test_cumsum_f32(gpu, shape, dim, comp):
    rows, cols = shape
    rng = np.random.default_rng(rows * 3 + cols)
    A = rng.standard_normal(rows * cols).astype(np.float32)
    got = host(gpu.cumulative("cumsum", to_dev(A), rows, cols, dim, compensated=comp))
    check_cumsum(got, A, rows, cols, dim, comp)


def test_cumsum_long_vector_reproducible(gpu):
    """A 2^24-element column: 2048 tiles chained through the look-back; bitwise reproducible."""
    n = 1 << 24
    x = torch.empty(n, device="cuda")
    gpu.fill_normal(x, 7)
    a = host(gpu.cumulative("cumsum", x, n, 1, 1))
    b = host(gpu.cumulative("cumsum", x, n, 1, 1))
    assert np.array_equal(a.view(np.uint32), b.view(np.uint32))
    check_cumsum(a, host(x), n, 1, 1, True)
    p = host(gpu.cumulative("cumsum", x, n, 1, 1, compensated=False))
    check_cumsum(p, host(x), n, 1, 1, False)


def test_cumsum_long_column_wide_range(gpu):
    """Tile carries across the look-back (16384-element tiles) over values of every
    scale: huge terms that cancel, subnormals, exact zeros.  The carries are exact,
    so the compensated cumsum stays within its FP64 bound; a sum that overflows
    reads inf from there on, and a NaN poisons every later element."""
    n = 9 * 16384 + 123
    rng = np.random.default_rng(21)
    A = rng.standard_normal(n).astype(np.float32)
    A[::997] *= np.float32(1e30)                 # huge terms
    A[1::997] = -A[::997][: len(A[1::997])]      # ... that cancel right after
    A[2::50] = np.float32(1e-40)                 # subnormals
    A[3::70] = np.float32(0.0)
    got = host(gpu.cumulative("cumsum", to_dev(A), n, 1, 1))
    check_cumsum(got, A, n, 1, 1, True)
    # overflow: a run of +max values past a tile boundary
    B = np.ones(n, np.float32)
    B[40000:40004] = np.float32(3.0e38)
    got = host(gpu.cumulative("cumsum", to_dev(B), n, 1, 1))
    assert np.all(np.isfinite(got[:40001])) and np.all(np.isposinf(got[40001:]))
    # a NaN in the third tile
    C = np.ones(n, np.float32)
    C[33000] = np.nan
    got = host(gpu.cumulative("cumsum", to_dev(C), n, 1, 1))
    assert np.array_equal(got[:33000], np.arange(1, 33001, dtype=np.float32))
    assert np.all(np.isnan(got[33000:]))


def test_cumsum_integer_valued_exact(gpu):
    # sums of small integers are exact in any order
    n = 1 << 20
    A = (np.arange(n) % 7).astype(np.float32)
    got = host(gpu.cumulative("cumsum", to_dev(A), n, 1, 1))
    assert np.array_equal(got, np.cumsum(A.astype(np.float64)).astype(np.float32))
    M = torch.arange(1, 13, dtype=torch.float32, device="cuda")     # 3x4 column-major
    assert host(gpu.cumulative("cumsum", M, 3, 4, 1)).tolist() == [1, 3, 6, 4, 9, 15, 7, 15, 24, 10, 21, 33]
    assert host(gpu.cumulative("cumsum", M, 3, 4, 2)).tolist() == [1, 2, 3, 5, 7, 9, 12, 15, 18, 22, 26, 30]


@pytest.mark.parametrize("shape", [(8192, 512), (1000, 3000)])
def test_cumsum_dim2_config(gpu, shape):
    rows, cols = shape
    Ad = torch.empty(rows * cols, device="cuda")
    gpu.fill_normal(Ad, 9)
    A = host(Ad)
    for dim in (1, 2):
        got = host(gpu.cumulative("cumsum", Ad, rows, cols, dim))
        check_cumsum(got, A, rows, cols, dim, True)
        again = host(gpu.cumulative("cumsum", Ad, rows, cols, dim))
        assert np.array_equal(got.view(np.uint32), again.view(np.uint32))


# Row scans of tables with at least one 128-byte strip of rows per SM take the
# TMA-staged single pass: ragged last strips (rows not a multiple of 32) and
# ragged last column tiles (cols not a multiple of 128), in place too.
@pytest.mark.parametrize("shape", [(4868, 130), (8192, 129), (4864, 1), (6000, 300)])
def test_row_scan_staged(gpu, shape):
    rows, cols = shape
    rng = np.random.default_rng(rows + cols)
    A = rng.standard_normal(rows * cols).astype(np.float32)
    for comp in (True, False):
        got = host(gpu.cumulative("cumsum", to_dev(A), rows, cols, 2, compensated=comp))
        check_cumsum(got, A, rows, cols, 2, comp)
    L = lines(A, rows, cols, 2)
    mx = back(np.maximum.accumulate(L, axis=1), rows, cols, 2).astype(np.float32)
    assert np.array_equal(host(gpu.cumulative("cummax", to_dev(A), rows, cols, 2)), mx)
    t = to_dev(A)
    gpu.cumulative("cumsum", t, rows, cols, 2, out=t)
    check_cumsum(host(t), A, rows, cols, 2, True)
    D = rng.standard_normal(rows * cols)
    got = host(gpu.cumulative("cumsum", to_dev(D), rows, cols, 2))
    LD = lines(D, rows, cols, 2)
    r = back(np.cumsum(LD, axis=1), rows, cols, 2)
    cabs = back(np.cumsum(np.abs(LD), axis=1), rows, cols, 2)
    assert np.all(np.abs(got - r) <= 128 * 2.0 ** -53 * cabs)


@pytest.mark.parametrize("shape", [(5, 3), (1000, 7), (20000, 2), (3, 5000)])
@pytest.mark.parametrize("dim", [1, 2])
def test_cumprod_f32(gpu, shape, dim):
    rows, cols = shape
    rng = np.random.default_rng(1)
    A = rng.uniform(0.999, 1.001, rows * cols).astype(np.float32)
    got = host(gpu.cumulative("cumprod", to_dev(A), rows, cols, dim)).astype(np.float64)
    L = lines(A, rows, cols, dim)
    r = back(np.cumprod(L, axis=1), rows, cols, dim)
    idx = back(np.broadcast_to(np.arange(L.shape[1]), L.shape), rows, cols, dim)
    assert np.all(np.abs(got - r) <= (idx + 16) * EPS * np.abs(r))


@pytest.mark.parametrize("shape", [(7, 3), (65, 5), (100003, 2), (3, 1000), (8192, 64)])
@pytest.mark.parametrize("dim", [1, 2])
def test_cummax_cummin_exact(gpu, shape, dim):
    rows, cols = shape
    rng = np.random.default_rng(rows + 5 * cols)
    A = rng.standard_normal(rows * cols).astype(np.float32)
    A[rng.integers(0, A.size, 4)] = np.nan
    L = lines(A, rows, cols, dim)
    mx = back(np.maximum.accumulate(np.where(np.isnan(L), -np.inf, L), axis=1), rows, cols, dim)
    mn = back(np.minimum.accumulate(np.where(np.isnan(L), np.inf, L), axis=1), rows, cols, dim)
    assert np.array_equal(host(gpu.cumulative("cummax", to_dev(A), rows, cols, dim)), mx.astype(np.float32))
    assert np.array_equal(host(gpu.cumulative("cummin", to_dev(A), rows, cols, dim)), mn.astype(np.float32))


def test_cumsum_in_place_and_overlap(gpu, cuda_lib):
    n = 50000
    rng = np.random.default_rng(3)
    A = rng.standard_normal(n).astype(np.float32)
    t = to_dev(A)
    gpu.cumulative("cumsum", t, n, 1, 1, out=t)
    check_cumsum(host(t), A, n, 1, 1, True)
    u = torch.zeros(n + 8, device="cuda")
    st = cuda_lib.nt2cuda_scan_f32(0, u.data_ptr(), n, 1, 1, u.data_ptr() + 16, 0,
                                   torch.cuda.current_stream().cuda_stream)
    assert st == 8   # NT2CUDA_ERR_ALIAS


def test_misaligned_views(gpu):
    rows, cols = 10001, 3
    rng = np.random.default_rng(8)
    base = to_dev(rng.standard_normal(rows * cols + 1).astype(np.float32))
    A = base[1:]
    out = torch.empty(rows * cols + 3, device="cuda")[3:]
    for dim in (1, 2):
        gpu.cumulative("cumsum", A, rows, cols, dim, out=out)
        check_cumsum(host(out), host(A), rows, cols, dim, True)


@pytest.mark.parametrize("dim", [1, 2])
def test_scans_f64(gpu, dim):
    rows, cols = 20000, 3
    rng = np.random.default_rng(4)
    A = rng.standard_normal(rows * cols)
    L = lines(A, rows, cols, dim)
    got = host(gpu.cumulative("cumsum", to_dev(A), rows, cols, dim))
    r = back(np.cumsum(L, axis=1), rows, cols, dim)
    cabs = back(np.cumsum(np.abs(L), axis=1), rows, cols, dim)
    assert np.all(np.abs(got - r) <= 128 * 2.0 ** -53 * cabs)
    mx = back(np.maximum.accumulate(L, axis=1), rows, cols, dim)
    assert np.array_equal(host(gpu.cumulative("cummax", to_dev(A), rows, cols, dim)), mx)


def test_no_wait_ran_out(cuda_lib):
    """No look-back wait of the scans above ran out."""
    import ctypes as C
    c = C.c_ulonglong(99)
    assert cuda_lib.nt2cuda_wait_timeouts(C.byref(c)) == 0
    assert c.value == 0


def test_wait_timeout_is_reported(gpu, cuda_lib):
    """A wait that nothing satisfies runs out (bounded polls, under a second), the kernel
    writes NaN over its tile and returns, the host reads NT2CUDA_ERR_TIMEOUT, and the context
    stays usable."""
    import ctypes as C
    c0, c1, c2 = C.c_ulonglong(), C.c_ulonglong(), C.c_ulonglong()
    assert cuda_lib.nt2cuda_wait_timeouts(C.byref(c0)) == 0
    st = cuda_lib.nt2cuda_selftest_wait_timeout(torch.cuda.current_stream().cuda_stream)
    assert st == 5                                        # NT2CUDA_ERR_TIMEOUT
    assert cuda_lib.nt2cuda_wait_timeouts(C.byref(c1)) == 0
    assert c1.value == c0.value + 1
    n = 1 << 20
    x = torch.empty(n, device="cuda")
    gpu.fill_normal(x, 11)
    check_cumsum(host(gpu.cumulative("cumsum", x, n, 1, 1)), host(x), n, 1, 1, True)
    assert cuda_lib.nt2cuda_wait_timeouts(C.byref(c2)) == 0
    assert c2.value == c1.value
