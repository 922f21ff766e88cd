"""Tables past 2^32 elements: every index is 64-bit (NT2's sizes are std::size_t).

saxpy is bit-exact against two separate torch operations (a*x rounded, then + y rounded, NT2's
unfused fma); the dot product and the long cumulative sum are held to their FP64 bounds; the
rows x cols reduction covers more than 2^32 elements in few columns.  Each test holds 16-33 GB of
device memory and frees it before the next one.
"""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

N = (1 << 32) + 37          # past 32-bit element counts, ragged against every vector width
EPS = 2.0 ** -24


def dsum(t, absolute=False):
    """FP64 sum of a float table, in chunks of 2^28 elements."""
    total = 0.0
    for k in range(0, t.numel(), 1 << 28):
        c = t[k:k + (1 << 28)].double()
        total += float((c.abs() if absolute else c).sum())
    return total


@pytest.fixture(autouse=True)
def _free():
    yield
    torch.cuda.synchronize()
    torch.cuda.empty_cache()


def test_saxpy_past_2_32(gpu):
    x = torch.empty(N, device="cuda")
    y = torch.empty(N, device="cuda")
    gpu.fill_uniform(x, -1.0, 1.0, 1)
    gpu.fill_uniform(y, -1.0, 1.0, 2)
    want = x * 2.5
    want += y
    gpu.saxpy(2.5, x, y)
    assert torch.equal(y.view(torch.int32), want.view(torch.int32))


def test_dot_past_2_32(gpu):
    x = torch.empty(N, device="cuda")
    y = torch.empty(N, device="cuda")
    gpu.fill_normal(x, 3)
    gpu.fill_normal(y, 4)
    got = float(gpu.dot(x, y).item())
    # FP64 reference of the float products, in chunks
    ref = 0.0
    aref = 0.0
    for k in range(0, N, 1 << 28):
        p = (x[k:k + (1 << 28)] * y[k:k + (1 << 28)]).double()
        ref += float(p.sum())
        aref += float(p.abs().sum())
    assert abs(got - ref) <= 8 * EPS * abs(ref) + 1e-9 * aref, (got, ref)


def test_cumsum_past_2_32(gpu):
    x = torch.empty(N, device="cuda")
    gpu.fill_uniform(x, 0.0, 1.0, 5)
    y = gpu.cumulative("cumsum", x, N, 1, 1)
    # checkpoints: the exact FP64 running sum at a few indices (compensated scan: 4 eps relative)
    idx = [0, 1, (1 << 31) - 1, 1 << 31, (1 << 32) - 1, 1 << 32, N - 1]
    run = 0.0
    prev = 0
    for i in idx:
        run += dsum(x[prev:i + 1])
        prev = i + 1
        got = float(y[i].item())
        assert abs(got - run) <= 4 * EPS * abs(run) + 64 * EPS * EPS * N * run, (i, got, run)


def test_column_sums_past_2_32(gpu):
    rows, cols = (1 << 31) + 5, 2                # 2^32 + 10 elements, two columns
    A = torch.empty(rows * cols, device="cuda")
    gpu.fill_uniform(A, -1.0, 1.0, 6)
    s = gpu.reduce("sum", A, rows, cols, 1)
    for j in range(cols):
        col = A[j * rows:(j + 1) * rows]
        ref = dsum(col)
        aref = dsum(col, absolute=True)
        assert abs(float(s[j].item()) - ref) <= 4 * EPS * abs(ref) + 1e-9 * aref, j
