"""Composed trigonometric functors on the GPU against the CPU oracle.

csc, sec, cscpi, secpi, cscd, cot, tanpi, cotpi and the degree forms sind,
cosd, tand, cotd, secd (in NT2's scalar form and its 128-bit pack form),
indeg, inrad, acot, asind, acosd, atand, asinpi, acospi, atanpi, acsc, acscd,
asec, asecd.  Exact mode (fused = 0) must be bit-identical to the oracle;
fused mode (hardware FMA in the polynomials) is held to the bounds below.
"""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

FORWARD = ["csc", "sec", "cscpi", "secpi", "cscd", "cot", "tanpi", "cotpi", "sind", "cosd", "tand", "cotd", "secd",
           "sinc", "sincpi"]
FAST = ["fast_sin", "fast_cos", "fast_tan", "fast_cot", "fast_sinpi", "fast_cospi", "fast_tanpi", "fast_cotpi",
        "fast_sind", "fast_cosd", "fast_tand", "fast_cotd", "proper_tanpi"]
INVERSE = ["indeg", "inrad", "acot", "asind", "acosd", "atand", "asinpi", "acospi", "atanpi", "acsc", "acscd",
           "asec", "asecd"]
SPECIALS = [0.0, -0.0, 1.0, -1.0, 0.5, -0.5, 2.0, 0.25, np.inf, -np.inf, np.nan, 180.0, -90.0, 45.0, 1e-30]
# fused (hardware FMA) against the exact oracle, ulpdist units: the reduction polynomials'
# bounds (2 scalar form, 8 pack form) plus the reciprocal's half ulp, on moderate ranges
FUSED_FORWARD = {False: 4.0, True: 16.0}
FUSED_INVERSE = 4.0


def to_dev(a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def host(t):
    torch.cuda.synchronize()
    return t.cpu().numpy()


def ref(oracle, op, x, pack=1):
    return oracle.trig(op, x, pack) if op in oracle.TRIG else oracle.trigx(op, x, pack)


def same_bits(y, ref):
    it = np.uint64 if y.dtype == np.float64 else np.uint32
    nan = np.isnan(y) & np.isnan(ref)
    return np.flatnonzero(~nan & (y.view(it) != ref.view(it)))


def inputs(op, n, dtype, seed):
    rng = np.random.default_rng(seed)
    if op in FORWARD:
        # every reduction level of sin/cos, and integers, halves and quarters for the pi forms
        hi = np.array([0.78, 1.57, 62.8, 201.0, 8.2e5, 1e30 if dtype == np.float32 else 1e200])
        x = rng.uniform(0, 1, n) * hi[rng.integers(0, hi.size, n)]
        x[::4] = np.round(x[::4] * 4) / 4
        if op in ("cscd", "sind", "cosd", "tand", "cotd", "secd"):
            x[1::4] = np.round(x[1::4] / 45) * 45
    elif op in FAST:
        # the fast forms' range and a margin beyond it (NaN there)
        r = 45.0 if op.endswith("d") else (0.5 if op == "proper_tanpi" else (0.25 if "pi" in op else 0.7854))
        x = rng.uniform(0, 1.2 * r, n)
    elif op in ("acsc", "acscd", "asec", "asecd", "acot"):
        x = np.exp(rng.uniform(-5, 8, n))
    elif op in ("indeg", "inrad"):
        x = np.exp(rng.uniform(-80, 80, n))
    elif op in ("atand", "atanpi"):
        x = np.exp(rng.uniform(-20, 20, n))
    else:
        x = rng.uniform(0, 1.2, n)
    x = (x * np.where(rng.integers(0, 2, n) == 1, -1.0, 1.0)).astype(dtype)
    k = min(n, len(SPECIALS))
    x[:k] = np.array(SPECIALS[:k], dtype)
    return x


@pytest.mark.parametrize("op", FORWARD)
@pytest.mark.parametrize("dtype", [np.float32, np.float64])
@pytest.mark.parametrize("simd", [False, True])
@pytest.mark.parametrize("n", [1, 7, 4097, (1 << 18) + 3])
def test_forward_bit_exact(gpu, oracle, op, dtype, simd, n):
    x = inputs(op, n, dtype, n)
    y = host(gpu.map_(op, to_dev(x), simd128=simd))
    pack = 16 // np.dtype(dtype).itemsize if simd else 1
    bad = same_bits(y, ref(oracle, op, x, pack))
    assert bad.size == 0, (op, dtype, simd, bad[:5], x[bad[:5]], y[bad[:5]])


@pytest.mark.parametrize("op", INVERSE + FAST)
@pytest.mark.parametrize("dtype", [np.float32, np.float64])
@pytest.mark.parametrize("n", [1, 7, 4097, (1 << 18) + 3])
def test_inverse_bit_exact(gpu, oracle, op, dtype, n):
    x = inputs(op, n, dtype, n + 1)
    y = host(gpu.map_(op, to_dev(x)))
    bad = same_bits(y, ref(oracle, op, x))
    assert bad.size == 0, (op, dtype, bad[:5], x[bad[:5]], y[bad[:5]])


@pytest.mark.parametrize("op", FORWARD + INVERSE + FAST)
@pytest.mark.parametrize("dtype", [np.float32, np.float64])
def test_fused_bound(gpu, oracle, op, dtype):
    rng = np.random.default_rng(6)
    n = 1 << 16
    if op in FORWARD:
        x = rng.uniform(-60, 60, n).astype(dtype)
        if op in ("cscd", "sind", "cosd", "tand", "cotd", "secd"):
            x = (x * 6).astype(dtype)
    else:
        x = inputs(op, n, dtype, 6)
    for simd in ((False, True) if op in FORWARD else (False,)):
        y = host(gpu.map_(op, to_dev(x), fused=True, simd128=simd))
        pack = 16 // np.dtype(dtype).itemsize if simd else 1
        m, w = oracle.max_ulp(y, ref(oracle, op, x, pack))
        bound = FUSED_FORWARD[simd] if op in FORWARD else FUSED_INVERSE
        assert m <= bound, (op, dtype, simd, m, x[w])


def test_misaligned_views(gpu, oracle):
    x = inputs("csc", 10001, np.float32, 3)
    d = to_dev(x)
    out = torch.empty(10001, device="cuda")
    for op in ("csc", "asecd"):
        for simd in (False, True):
            gpu.map_(op, d[1:], out=out[1:], simd128=simd and op == "csc")
            # an unaligned table takes NT2's scalar code throughout, in both forms
            assert same_bits(host(out)[1:], oracle.trigx(op, x[1:])).size == 0, (op, simd)


SINCOS = {"sincos": ("sin", "cos"), "sincospi": ("sinpi", "cospi"), "sincosd": ("sind", "cosd"),
          "fast_sincos": ("fast_sin", "fast_cos"), "fast_sincospi": ("fast_sinpi", "fast_cospi"),
          "fast_sincosd": ("fast_sind", "fast_cosd"), "sinhcosh": ("sinh", "cosh")}


@pytest.mark.parametrize("form", sorted(SINCOS))
@pytest.mark.parametrize("dtype", [np.float32, np.float64])
@pytest.mark.parametrize("simd", [False, True])
def test_sincos_pairs(gpu, oracle, form, dtype, simd):
    """tie(s, c) = sincos(x) in one pass equals (sin(x), cos(x)) of the same form, bit for bit
    (NT2's sincosa takes the reduction and the signs sina and cosa take)."""
    sname, cname = SINCOS[form]
    x = inputs(sname, 65537, dtype, 8) if form != "sinhcosh" else \
        np.random.default_rng(8).uniform(-100, 100, 65537).astype(dtype)
    s, c = gpu.sincos(to_dev(x), form=form, simd128=simd)
    pack = 16 // np.dtype(dtype).itemsize if simd and form in ("sincos", "sincospi", "sincosd") else 1
    if form == "sinhcosh":
        sref, cref = oracle.map_("sinh", x), oracle.map_("cosh", x)
    else:
        sref, cref = ref(oracle, sname, x, pack), ref(oracle, cname, x, pack)
    assert same_bits(host(s), sref).size == 0, (form, "sin")
    assert same_bits(host(c), cref).size == 0, (form, "cos")
