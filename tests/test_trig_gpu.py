"""sin, cos, tan, sinpi, cospi on the GPU against the CPU oracle.

Exact mode (fused = 0) must be bit-identical to the oracle in both forms:
NT2's scalar code (each element reduced on its own, the default) and NT2's
128-bit SIMD code (NT2CUDA_MAP_SIMD128: one reduction method per 16-byte pack,
chosen from the pack's largest |x|; scalar tail).  The inputs mix every
reduction level in and across packs: |x| <= pi/4, <= pi/2, <= 20 pi,
<= Medium_pi, <= 2^18 pi and beyond (fdlibm's range and the exact reduction),
plus NaN, +-Inf and signed zeros.  Fused mode (hardware FMA in the
polynomials) is held to 2 ulpdist units of the oracle on NT2's cover ranges
(8 in the 128-bit form, see test_trig_fused_bound).
"""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

OPS = ["sin", "cos", "tan", "sinpi", "cospi"]
COVER = {"sin": 60.0, "cos": 60.0, "tan": 60.0, "sinpi": 40.0, "cospi": 41.0}
SPECIALS = [0.0, -0.0, np.inf, -np.inf, np.nan, np.pi / 2, -np.pi / 4, np.pi, 1e-30, 823549.6875, 201.0625, 1e22]


def to_dev(a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def host(t):
    torch.cuda.synchronize()
    return t.cpu().numpy()


def mixed(n, dtype, seed):
    """Each element drawn from one reduction level's range (levels vary within packs)."""
    rng = np.random.default_rng(seed)
    hi = [0.78, 1.57, 62.8, 201.0, 823549.0, 1e30 if dtype == np.float32 else 1e300]
    lv = rng.integers(0, len(hi), n)
    u = rng.uniform(0, 1, n)
    x = np.where(lv < 4, u * np.take(hi, np.minimum(lv, 3)),
                 10.0 ** (5.9 + u * (np.log10(np.take(hi, np.maximum(lv, 4))) - 5.9)))
    x = np.where(rng.integers(0, 2, n) == 1, -x, x).astype(dtype)
    # whole packs of one level too (the common case)
    if n >= 64:
        for k in range(6):
            x[8 * k: 8 * k + 8] = (rng.uniform(0, 1, 8) * (hi[k] if k < 4 else 1.0) + (0 if k < 4 else hi[k - 1])
                                   ).astype(dtype)
    if n >= 64 + len(SPECIALS):
        x[64: 64 + len(SPECIALS)] = np.array(SPECIALS).astype(dtype)
    return x


def same_bits(y, ref):
    nan = np.isnan(y) & np.isnan(ref)
    bad = ~nan & (y.view(np.uint64 if y.dtype == np.float64 else np.uint32)
                  != ref.view(np.uint64 if ref.dtype == np.float64 else np.uint32))
    return np.flatnonzero(bad)


@pytest.mark.parametrize("op", OPS)
@pytest.mark.parametrize("dtype", [np.float32, np.float64])
@pytest.mark.parametrize("n", [0, 1, 3, 5, 8, 97, (1 << 18) + 3])
def test_trig_bit_exact_scalar_form(gpu, oracle, op, dtype, n):
    x = mixed(n, dtype, seed=n + 7)
    y = host(gpu.map_(op, to_dev(x)))
    bad = same_bits(y, oracle.trig(op, x, 1))
    assert bad.size == 0, (op, dtype, bad[:5], x[bad[:5]], y[bad[:5]])


@pytest.mark.parametrize("op", OPS)
@pytest.mark.parametrize("dtype", [np.float32, np.float64])
@pytest.mark.parametrize("n", [1, 3, 5, 8, 97, (1 << 18) + 3])
def test_trig_bit_exact_simd128_form(gpu, oracle, op, dtype, n):
    x = mixed(n, dtype, seed=n + 11)
    y = host(gpu.map_(op, to_dev(x), simd128=True))
    pack = 16 // np.dtype(dtype).itemsize
    bad = same_bits(y, oracle.trig(op, x, pack))
    assert bad.size == 0, (op, dtype, bad[:5], x[bad[:5]], y[bad[:5]])


@pytest.mark.parametrize("dtype", [np.float32, np.float64])
def test_trig_simd128_misaligned_is_scalar(gpu, oracle, dtype):
    n = 10001
    x = mixed(n + 1, dtype, seed=3)
    xd = to_dev(x)[1:]
    out = torch.empty(n + 1, dtype=xd.dtype, device="cuda")[1:]
    for op in OPS:
        gpu.map_(op, xd, out=out, simd128=True)
        assert same_bits(host(out), oracle.trig(op, x[1:], 1)).size == 0, op


def test_trig_in_place(gpu, oracle):
    x = mixed(4099, np.float32, seed=5)
    t = to_dev(x)
    gpu.map_("sin", t, out=t, simd128=True)
    assert same_bits(host(t), oracle.trig("sin", x, 4)).size == 0
    t = to_dev(x)
    gpu.map_("cos", t, out=t)
    assert same_bits(host(t), oracle.trig("cos", x, 1)).size == 0


@pytest.mark.parametrize("op", OPS)
@pytest.mark.parametrize("dtype", [np.float32, np.float64])
def test_trig_fused_bound(gpu, oracle, op, dtype):
    lim = COVER[op]
    x = np.random.default_rng(9).uniform(-lim, lim, 200003).astype(dtype)
    # 128-bit packs reduce a lane under pi/4 by x - pi/2 when a neighbour lies in (pi/4, pi/2]; the
    # polynomial then cancels and magnifies the contraction's rounding difference a few times
    for simd, bound in ((False, 2.0), (True, 8.0)):
        y = host(gpu.map_(op, to_dev(x), fused=True, simd128=simd))
        ref = oracle.trig(op, x, 16 // np.dtype(dtype).itemsize if simd else 1)
        m, w = oracle.max_ulp(y, ref)
        assert m <= bound, (op, dtype, simd, m, x[w])


def test_trig_table_sizes_large(gpu, oracle):
    """A 2^24-element table (one full grid of persistent blocks, several trips)."""
    n = 1 << 24
    x = torch.empty(n, device="cuda")
    gpu.fill_uniform(x, -60.0, 60.0, 13)
    y = host(gpu.map_("sin", x))
    xs = host(x)
    idx = np.random.default_rng(1).integers(0, n, 200000)
    assert same_bits(y[idx], oracle.trig("sin", np.ascontiguousarray(xs[idx]), 1)).size == 0


INV = {"asin": 1.2, "acos": 1.2, "atan": 1e4}


@pytest.mark.parametrize("op", sorted(INV))
@pytest.mark.parametrize("dtype", [np.float32, np.float64])
@pytest.mark.parametrize("n", [0, 1, 5, 97, (1 << 18) + 3])
def test_invtrig_bit_exact(gpu, oracle, op, dtype, n):
    """asin, acos, atan: NT2's SIMD forms element by element, bit-exact (NaN beyond [-1, 1])."""
    rng = np.random.default_rng(n + 3)
    lim = INV[op]
    x = rng.uniform(-lim, lim, n)
    if op == "atan" and n > 8:
        x[: n // 2] = np.tan(rng.uniform(-1.5, 1.5, n // 2))
    x = x.astype(dtype)
    if n >= 64:
        x[:12] = np.array([0.0, -0.0, 0.5, -0.5, 1.0, -1.0, np.inf, -np.inf, np.nan, 0.625, 0.41421356,
                           2.4142135], dtype)
    y = host(gpu.map_(op, to_dev(x)))
    bad = same_bits(y, oracle.trig(op, x))
    assert bad.size == 0, (op, dtype, bad[:5], x[bad[:5]], y[bad[:5]])
    # the 128-bit flag changes nothing for the inverse functions
    if n:
        y2 = host(gpu.map_(op, to_dev(x), simd128=True))
        assert same_bits(y2, y).size == 0


@pytest.mark.parametrize("op", sorted(INV))
@pytest.mark.parametrize("dtype", [np.float32, np.float64])
def test_invtrig_fused_bound(gpu, oracle, op, dtype):
    x = np.random.default_rng(2).uniform(-INV[op], INV[op], 100003).astype(dtype)
    y = host(gpu.map_(op, to_dev(x), fused=True))
    m, w = oracle.max_ulp(y, oracle.trig(op, x))
    assert m <= 2.0, (op, dtype, m, x[w])


@pytest.mark.parametrize("dtype", [np.float32, np.float64])
@pytest.mark.parametrize("n", [1, 7, 100, (1 << 18) + 3])
def test_atan2_bit_exact(gpu, oracle, dtype, n):
    rng = np.random.default_rng(n)
    a = rng.uniform(-3, 3, n).astype(dtype)
    b = rng.uniform(-3, 3, n).astype(dtype)
    if n >= 100:
        sp = np.array([0.0, -0.0, 1.0, -1.0, np.inf, -np.inf, np.nan, 0.5, 1e-30, 3e30], dtype)
        a[:100] = np.repeat(sp, 10)
        b[:100] = np.tile(sp, 10)
    y = host(gpu.atan2(to_dev(a), to_dev(b)))
    bad = same_bits(y, oracle.atan2(a, b))
    assert bad.size == 0, (dtype, bad[:5], a[bad[:5]], b[bad[:5]], y[bad[:5]])
    yf = host(gpu.atan2(to_dev(a), to_dev(b), fused=True))
    m, w = oracle.max_ulp(yf, oracle.atan2(a, b))
    assert m <= 2.0, (dtype, m, a[w], b[w])
