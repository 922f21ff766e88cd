"""The NT2 evaluation site (include/nt2/sdk/cuda/eval.hpp) lowers NT2's Proto
trees through nt2cuda/table_lowering.hpp and runs them through
nt2cuda/site.hpp.  Boost is absent here, so tests/site/nt2_site_mock.cu builds
trees of the same shape from NT2's own functor tags and calls the same site
operations; their results must equal the oracle's (bit for bit for the
elementwise statements, within the fold bounds for the reductions)."""
import os
import subprocess
import sys

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
EPS = 2.0 ** -24


@pytest.fixture(scope="module")
def mock(cuda_lib):
    sys.path.insert(0, os.path.join(HERE, "site"))
    import build_site_mock
    return build_site_mock.build()


def run(mock, args):
    r = subprocess.run([mock, *map(str, args)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr


def save(tmp_path, name, a):
    p = tmp_path / name
    a.tofile(p)
    return p


def test_saxpy_tree(mock, oracle, tmp_path):
    n = (1 << 20) + 7
    rng = np.random.default_rng(3)
    x = rng.uniform(-1, 1, n).astype(np.float32)
    y = rng.uniform(-1, 1, n).astype(np.float32)
    out = tmp_path / "out"
    run(mock, ["saxpy", n, 2.5, save(tmp_path, "x", x), save(tmp_path, "y", y), out])
    ref = y.copy()
    oracle.load().nt2o_saxpy_f(2.5, x, ref, n, 0)
    assert np.array_equal(np.fromfile(out, np.float32).view(np.uint32), ref.view(np.uint32))


def test_transform_range(mock, oracle, tmp_path):
    """NT2's transform_ hands the site a (begin, size) range: only that range is written."""
    n, begin, size = 10007, 1001, 5003
    rng = np.random.default_rng(4)
    x = rng.uniform(-1, 1, n).astype(np.float32)
    y = rng.uniform(-1, 1, n).astype(np.float32)
    out = tmp_path / "out"
    run(mock, ["range", n, begin, size, -1.25, save(tmp_path, "x", x), save(tmp_path, "y", y), out])
    ref = y.copy()
    part = ref[begin:begin + size].copy()
    oracle.load().nt2o_saxpy_f(-1.25, np.ascontiguousarray(x[begin:begin + size]), part, size, 0)
    ref[begin:begin + size] = part
    assert np.array_equal(np.fromfile(out, np.float32).view(np.uint32), ref.view(np.uint32))


def test_blackscholes_trees(mock, oracle, tmp_path):
    n = (1 << 18) + 3
    rng = np.random.default_rng(5)
    S = rng.uniform(5, 30, n).astype(np.float32)
    K = rng.uniform(1, 100, n).astype(np.float32)
    T = rng.uniform(0.25, 10, n).astype(np.float32)
    oc, op = tmp_path / "call", tmp_path / "put"
    run(mock, ["bs", n, 0.02, 0.30, save(tmp_path, "S", S), save(tmp_path, "K", K), save(tmp_path, "T", T), oc, op])
    rc, rp = oracle.bs(S, K, T, 0.02, 0.30)
    assert np.array_equal(np.fromfile(oc, np.float32).view(np.uint32), rc.view(np.uint32))
    assert np.array_equal(np.fromfile(op, np.float32).view(np.uint32), rp.view(np.uint32))


def test_sdot_through_inner_fold(mock, oracle, tmp_path):
    n = (1 << 22) + 5
    rng = np.random.default_rng(6)
    x = rng.standard_normal(n).astype(np.float32)
    y = rng.standard_normal(n).astype(np.float32)
    out = tmp_path / "out"
    run(mock, ["sdot", n, save(tmp_path, "x", x), save(tmp_path, "y", y), out])
    ref, ab = oracle.dot_fp64(x, y)
    got = float(np.fromfile(out, np.float32)[0])
    assert abs(got - ref) <= 4 * EPS * abs(ref) + 64 * EPS * EPS * n * ab + EPS * ab


def test_row_sums_through_outer_fold(mock, oracle, tmp_path):
    rows, cols = 4099, 257
    rng = np.random.default_rng(7)
    A = rng.standard_normal(rows * cols).astype(np.float32)
    out = tmp_path / "out"
    run(mock, ["rowsum", rows, cols, save(tmp_path, "A", A), out])
    _, r64, ab = oracle.outer_fold(A, rows, cols)
    got = np.fromfile(out, np.float32).astype(np.float64)
    assert np.all(np.abs(got - r64) <= 4 * EPS * np.abs(r64) + 64 * EPS * EPS * cols * ab)
