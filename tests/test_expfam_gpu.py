"""The rest of NT2's exponential family on the GPU against the CPU oracle.

Unary (nt2cuda_map_*): cbrt, sqrt1pm1, exprecneg, exprecnegc, expx2, realsqrt,
reallog.  Binary (nt2cuda_map2_*): atan2, pow, pow_abs, realpow, logspace_add,
logspace_sub, expx2(x, s).  Exact mode (fused = 0) is bit-identical to the
oracle on inputs spread over the whole exponent range plus zeros, infinities,
NaN and denormals; fused mode (hardware FMA) is held to the bounds below.
"""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

UNARY = ["cbrt", "sqrt1pm1", "exprecneg", "exprecnegc", "expx2", "realsqrt", "reallog", "atanh", "acosh", "sech",
         "csch", "acoth", "asech", "asinh", "acsch", "coth", "sinhc"]
BINARY = ["atan2", "pow", "pow_abs", "realpow", "logspace_add", "logspace_sub", "expx2", "atan2d", "nbd_atan2", "hypot"]
SPECIALS = [0.0, -0.0, 1.0, -1.0, 0.5, -0.5, 8.0, -27.0, np.inf, -np.inf, np.nan, 1e-40, -1e-40, 88.7, 9.5]
# fused mode against the exact oracle, ulpdist units, on [-10, 10] (measured maxima: 2, 0, 2, 4, 2 and
# 2, 4 for pow_abs, expx2(x, s)); logspace_add and logspace_sub are checked in absolute terms (a few
# eps of max(|a0|, |a1|, 1)) because they cancel where their result is near zero
FUSED_BOUND = {"cbrt": 2.0, "sqrt1pm1": 0.0, "exprecneg": 2.0, "exprecnegc": 4.0, "expx2": 2.0,
               "realsqrt": 0.0, "reallog": 1.0, "atanh": 4.0, "acosh": 4.0, "sech": 4.0, "csch": 4.0, "acoth": 4.0,
               "asech": 4.0, "asinh": 4.0, "acsch": 4.0, "coth": 4.0, "sinhc": 4.0}
FUSED_BOUND2 = {"pow_abs": 2.0, "realpow": 2.0, "pow": 2.0, "expx2": 4.0, "atan2": 2.0, "atan2d": 4.0, "nbd_atan2": 2.0, "hypot": 0.0}


def to_dev(a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def host(t):
    torch.cuda.synchronize()
    return t.cpu().numpy()


def same_bits(y, ref):
    it = np.uint64 if y.dtype == np.float64 else np.uint32
    nan = np.isnan(y) & np.isnan(ref)
    return np.flatnonzero(~nan & (y.view(it) != ref.view(it)))


def wide(n, dtype, seed):
    """Signed values over the type's exponent range, the specials first."""
    rng = np.random.default_rng(seed)
    lim = 85.0 if dtype == np.float32 else 700.0
    x = (np.where(rng.integers(0, 2, n) == 1, -1.0, 1.0) * np.exp(rng.uniform(-lim, lim, n))).astype(dtype)
    x[: n // 3] = rng.uniform(-10, 10, n // 3).astype(dtype)
    k = min(n, len(SPECIALS))
    x[:k] = np.array(SPECIALS[:k], dtype)
    return x


@pytest.mark.parametrize("op", UNARY)
@pytest.mark.parametrize("dtype", [np.float32, np.float64])
@pytest.mark.parametrize("n", [1, 17, 4097, (1 << 18) + 3])
def test_unary_bit_exact(gpu, oracle, op, dtype, n):
    x = wide(n, dtype, n)
    y = host(gpu.map_(op, to_dev(x)))
    bad = same_bits(y, oracle.map_(op, x))
    assert bad.size == 0, (op, dtype, bad[:5], x[bad[:5]], y[bad[:5]])


@pytest.mark.parametrize("op", BINARY)
@pytest.mark.parametrize("dtype", [np.float32, np.float64])
@pytest.mark.parametrize("n", [1, 17, 4097, (1 << 18) + 3])
def test_binary_bit_exact(gpu, oracle, op, dtype, n):
    rng = np.random.default_rng(n + 7)
    a0 = rng.uniform(-30, 30, n).astype(dtype)
    a1 = rng.uniform(-30, 30, n).astype(dtype)
    a1[::5] = a0[::5] + dtype(1e-3)                  # near-equal pairs (logspace_sub's small branch)
    if op in ("pow", "pow_abs", "realpow"):
        a0 = np.abs(a0) * np.where(rng.integers(0, 4, n) == 0, -1, 1).astype(dtype)
        a1[1::3] = np.round(a1[1::3])                # integer exponents for negative bases
    if n >= len(SPECIALS) ** 2:
        sp = np.array(SPECIALS, dtype)
        a0[: sp.size ** 2] = np.repeat(sp, sp.size)
        a1[: sp.size ** 2] = np.tile(sp, sp.size)
    y = host(gpu.map2(op, to_dev(a0), to_dev(a1)))
    bad = same_bits(y, oracle.map2(op, a0, a1))
    assert bad.size == 0, (op, dtype, bad[:5], a0[bad[:5]], a1[bad[:5]], y[bad[:5]])


@pytest.mark.parametrize("op", UNARY)
@pytest.mark.parametrize("dtype", [np.float32, np.float64])
def test_unary_fused_bound(gpu, oracle, op, dtype):
    x = np.random.default_rng(3).uniform(-10, 10, 1 << 16).astype(dtype)
    if op in ("realsqrt", "reallog"):
        x = np.abs(x)
    y = host(gpu.map_(op, to_dev(x), fused=True))
    m, w = oracle.max_ulp(y, oracle.map_(op, x))
    assert m <= FUSED_BOUND[op], (op, dtype, m, x[w])


@pytest.mark.parametrize("op", BINARY)
@pytest.mark.parametrize("dtype", [np.float32, np.float64])
def test_binary_fused_bound(gpu, oracle, op, dtype):
    rng = np.random.default_rng(4)
    a0 = rng.uniform(0 if "pow" in op else -10, 10, 1 << 16).astype(dtype)
    a1 = rng.uniform(-10, 10, 1 << 16).astype(dtype)
    y = host(gpu.map2(op, to_dev(a0), to_dev(a1), fused=True))
    ref = oracle.map2(op, a0, a1)
    if op.startswith("logspace"):
        eps = float(np.finfo(dtype).eps)
        scale = np.maximum(np.maximum(np.abs(a0), np.abs(a1)), 1.0).astype(np.float64)
        same = (y == ref) | (np.isnan(y) & np.isnan(ref))   # NaN: log of a negative difference
        err = np.where(same, 0.0, np.abs(y.astype(np.float64) - ref.astype(np.float64)))
        bound = 4.0 if op == "logspace_add" else 8.0
        assert (err <= bound * eps * scale).all(), (op, dtype, float((err / scale).max() / eps))
    else:
        m, w = oracle.max_ulp(y, ref)
        assert m <= FUSED_BOUND2[op], (op, dtype, m, a0[w], a1[w])


def test_misaligned_views(gpu, oracle):
    """Tables one element past a 16-byte boundary take the unaligned path."""
    x = wide(10001, np.float32, 9)
    z = wide(10001, np.float32, 10)
    dx, dz = to_dev(x), to_dev(z)
    out = torch.empty(10001, device="cuda")
    gpu.map_("cbrt", dx[1:], out=out[1:])
    assert same_bits(host(out)[1:], oracle.map_("cbrt", x[1:])).size == 0
    gpu.map2("logspace_add", dx[1:], dz[1:], out=out[1:])
    assert same_bits(host(out)[1:], oracle.map2("logspace_add", x[1:], z[1:])).size == 0


def test_map2_arguments(cuda_lib):
    L = cuda_lib
    x = torch.ones(4, device="cuda")
    s = torch.cuda.current_stream().cuda_stream
    p = x.data_ptr()
    assert L.nt2cuda_map2_f32(42, p, p, p, 4, 0, s) != 0          # unknown functor
    assert L.nt2cuda_map2_f32(4, p, p, p, 4, 2, s) != 0           # SIMD128 is not a map2 flag
    assert L.nt2cuda_map2_f64(4, None, p, p, 4, 0, s) != 0        # null table
    assert L.nt2cuda_map2_f32(4, p, p, p, 0, 0, s) == 0           # empty tables
