"""pow(a0, a1) on the GPU against the CPU oracle (NT2's SIMD pow, floating exponents).

Exact mode (fused = 0) must be bit-identical to the oracle: NT2's cover range
(a0 in [0, 100], a1 in [-10, 10]), bases over the whole exponent range with
integer and fractional exponents, negative bases (odd and even integer
exponents, NaN otherwise), results that underflow into denormals or overflow,
denormal bases, and every pair of the special values.  Fused mode (hardware
FMA in NT2's fma steps and polynomials) is held to 2 ulpdist units of the
oracle on the cover range.
"""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

SPECIALS = [0.0, -0.0, 1.0, -1.0, 2.0, 0.5, -2.0, np.inf, -np.inf, np.nan, 1e-40, 3.0, -3.0, 2.5, 127.9,
            149.0, -149.0, 1025.0, -1075.0, 1e30]


def to_dev(a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def host(t):
    torch.cuda.synchronize()
    return t.cpu().numpy()


def same_bits(y, ref):
    it = np.uint64 if y.dtype == np.float64 else np.uint32
    nan = np.isnan(y) & np.isnan(ref)
    return np.flatnonzero(~nan & (y.view(it) != ref.view(it)))


def inputs(n, dtype, seed):
    rng = np.random.default_rng(seed)
    kind = rng.integers(0, 4, n)
    big = 80.0 if dtype == np.float32 else 700.0
    a0 = np.where(kind == 0, rng.uniform(0, 100, n),
                  np.where(kind == 1, np.exp(rng.uniform(-big, big, n)), -np.exp(rng.uniform(-big, big, n))))
    a1 = np.where(kind == 0, rng.uniform(-10, 10, n), rng.uniform(-3, 3, n))
    a1 = np.where(kind >= 2, np.round(rng.uniform(-40, 40, n)), a1)     # integer exponents: negative bases
    a1 = np.where(kind == 3, a1 + 0.5 * (rng.integers(0, 4, n) == 0), a1)  # ... and a few that are not
    a0, a1 = a0.astype(dtype), a1.astype(dtype)
    if n >= 500:
        sp = np.array(SPECIALS, dtype)
        k = len(sp)
        a0[:k * k] = np.repeat(sp, k)
        a1[:k * k] = np.tile(sp, k)
    return a0, a1


@pytest.mark.parametrize("dtype", [np.float32, np.float64])
@pytest.mark.parametrize("n", [1, 7, 1000, 65537, 1 << 20])
def test_pow_bit_exact(gpu, oracle, dtype, n):
    a0, a1 = inputs(n, dtype, n)
    y = host(gpu.pow(to_dev(a0), to_dev(a1)))
    bad = same_bits(y, oracle.pow_(a0, a1))
    assert bad.size == 0, (dtype, bad[:5], a0[bad[:5]], a1[bad[:5]], y[bad[:5]])


@pytest.mark.parametrize("dtype", [np.float32, np.float64])
def test_pow_misaligned_views(gpu, oracle, dtype):
    """Tables that start one element past a 16-byte boundary take the unaligned path."""
    a0, a1 = inputs(10001, dtype, 5)
    d0, d1 = to_dev(a0), to_dev(a1)
    out = torch.empty(10001, dtype=d0.dtype, device="cuda")
    gpu.pow(d0[1:], d1[1:], out=out[1:])
    y = host(out)[1:]
    bad = same_bits(y, oracle.pow_(a0[1:], a1[1:]))
    assert bad.size == 0, (dtype, bad[:5])


@pytest.mark.parametrize("dtype", [np.float32, np.float64])
def test_pow_fused_bound(gpu, oracle, dtype):
    rng = np.random.default_rng(3)
    n = 1 << 18
    a0 = rng.uniform(0, 100, n).astype(dtype)
    a1 = rng.uniform(-10, 10, n).astype(dtype)
    y = host(gpu.pow(to_dev(a0), to_dev(a1), fused=True))
    m, w = oracle.max_ulp(y, oracle.pow_(a0, a1))
    assert m <= 2.0, (dtype, m, a0[w], a1[w])


def test_pow_flags_rejected(cuda_lib):
    x = torch.ones(4, device="cuda")
    s = torch.cuda.current_stream().cuda_stream
    assert cuda_lib.nt2cuda_pow_f32(x.data_ptr(), x.data_ptr(), x.data_ptr(), 4, 2, s) != 0
    assert cuda_lib.nt2cuda_pow_f32(x.data_ptr(), x.data_ptr(), x.data_ptr(), 0, 0, s) == 0
