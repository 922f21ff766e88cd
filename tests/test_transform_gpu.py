"""Elementwise statements on the GPU against the CPU oracle.

With fused = 0 the device evaluates NT2's arithmetic with the same
roundings as the oracle, so every float32/float64 result must be
bit-identical (ulpdist 0; NaNs compare equal).  fused = 1 (hardware FMA) is
held to the stated ULP bounds below.
"""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

SIZES = [0, 1, 3, 7, 31, 33, 1000, 4097, (1 << 16) + 5]
# fused-FMA bounds (NT2 ulpdist units) against the unfused oracle; erfc and normcdf stay within
# the 16 ULP that NT2 states for its float erfc (erf_kernel.hpp:50-52)
FUSED_BOUND = {"exp": 1.0, "log": 1.0, "erfc": 16.0, "normcdf": 16.0, "fastnormcdf": 8.0, "sqrt": 0.0,
               "exp2": 2.0, "exp10": 2.0, "log2": 2.0, "log10": 2.0, "expm1": 2.0, "log1p": 2.0,
               "sinh": 2.0, "cosh": 2.0, "tanh": 2.0}


def to_dev(a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def host(t):
    torch.cuda.synchronize()
    return t.cpu().numpy()


def inputs(op, n, dtype, seed=0):
    rng = np.random.default_rng(seed)
    if op in ("log", "sqrt", "log2", "log10"):
        x = rng.uniform(0, 100, n)
    elif op == "exp":
        x = rng.uniform(-100, 100, n)
    elif op == "exp2":
        x = rng.uniform(-150, 150, n)
    elif op == "exp10":
        x = rng.uniform(-45, 45, n)
    elif op == "expm1":
        x = rng.uniform(-100, 100, n)
    elif op == "log1p":
        x = rng.uniform(-1, 100, n)
    else:
        x = rng.uniform(-10, 10, n)
    x = x.astype(dtype)
    specials = np.array([0.0, -0.0, 1.0, -1.0, np.inf, -np.inf, np.nan, 88.5, -88.5, 1e-40, -3.0], dtype)
    if n >= len(specials):
        x[: len(specials)] = specials
    return x


@pytest.mark.parametrize("op", ["exp", "log", "erfc", "normcdf", "fastnormcdf", "sqrt", "exp2", "exp10", "log2",
                                "log10", "expm1", "log1p", "sinh", "cosh", "tanh"])
@pytest.mark.parametrize("n", SIZES)
def test_map_f32_bit_exact(gpu, oracle, op, n):
    x = inputs(op, n, np.float32, seed=n)
    y = host(gpu.map_(op, to_dev(x)))
    ref = oracle.map_(op, x)
    m, w = oracle.max_ulp(y, ref)
    assert m == 0.0, (op, n, w, x[w] if n else None, y[w] if n else None, ref[w] if n else None)


@pytest.mark.parametrize("op", ["exp", "log", "erfc", "normcdf", "sqrt", "exp2", "exp10", "log2", "log10", "expm1",
                                "log1p", "sinh", "cosh", "tanh"])
@pytest.mark.parametrize("n", [1, 7, 4097, (1 << 16) + 3])
def test_map_f64_bit_exact(gpu, oracle, op, n):
    x = inputs(op, n, np.float64, seed=n + 1)
    y = host(gpu.map_(op, to_dev(x)))
    ref = oracle.map_(op, x)
    m, w = oracle.max_ulp(y, ref)
    assert m == 0.0, (op, n, w)


@pytest.mark.parametrize("op", ["exp", "log", "erfc", "normcdf", "fastnormcdf", "exp2", "exp10", "log2", "log10",
                                "expm1", "log1p", "sinh", "cosh", "tanh"])
def test_map_f32_fused_within_bound(gpu, oracle, op):
    x = inputs(op, 1 << 16, np.float32, seed=5)
    y = host(gpu.map_(op, to_dev(x), fused=True))
    m, _ = oracle.max_ulp(y, oracle.map_(op, x))
    assert m <= FUSED_BOUND[op], (op, m)


def test_map_misaligned_views(gpu, oracle):
    x = inputs("erfc", 1000, np.float32)
    xd = to_dev(x)
    out = torch.empty(1000, dtype=torch.float32, device="cuda")
    for off in (1, 2, 3):
        xv = xd[off:]
        yv = out[off:]
        gpu.map_("erfc", xv, out=yv)
        m, _ = oracle.max_ulp(host(yv), oracle.map_("erfc", x[off:]))
        assert m == 0.0


@pytest.mark.parametrize("n", SIZES)
@pytest.mark.parametrize("dtype", [np.float32, np.float64])
def test_saxpy_bit_exact(gpu, oracle, n, dtype):
    rng = np.random.default_rng(n)
    x = rng.uniform(-1, 1, n).astype(dtype)
    y = rng.uniform(-1, 1, n).astype(dtype)
    yd = to_dev(y)
    gpu.saxpy(2.5, to_dev(x), yd)
    ref = y.copy()
    (oracle.load().nt2o_saxpy_f if dtype == np.float32 else oracle.load().nt2o_saxpy_d)(2.5, x, ref, n, 1)
    assert np.array_equal(host(yd).view(np.uint8), ref.view(np.uint8))


def test_rgb2grey_bit_exact(gpu, oracle):
    n = 1920 * 1080 + 3
    rng = np.random.default_rng(9)
    r, g, b = (rng.uniform(0, 255, n).astype(np.float32) for _ in range(3))
    out = host(gpu.rgb2grey(to_dev(r), to_dev(g), to_dev(b)))
    ref = np.empty_like(r)
    oracle.load().nt2o_rgb2grey_f(r, g, b, ref, n, 1)
    assert np.array_equal(out.view(np.uint32), ref.view(np.uint32))


def bs_inputs(n, dtype, seed=42):
    rng = np.random.default_rng(seed)
    S = rng.uniform(5, 30, n).astype(dtype)
    K = rng.uniform(1, 100, n).astype(dtype)
    T = rng.uniform(0.25, 10, n).astype(dtype)
    return S, K, T


@pytest.mark.parametrize("cdf", ["normcdf", "fastnormcdf"])
@pytest.mark.parametrize("n", [1, 5, 1023, 4099, 1 << 20])
def test_blackscholes_f32_bit_exact(gpu, oracle, cdf, n):
    S, K, T = bs_inputs(n, np.float32, seed=n)
    c, p = gpu.blackscholes(to_dev(S), to_dev(K), to_dev(T), 0.02, 0.30, cdf=cdf)
    rc, rp = oracle.bs(S, K, T, 0.02, 0.30, cdf=0 if cdf == "normcdf" else 1)
    for got, ref in ((host(c), rc), (host(p), rp)):
        m, w = oracle.max_ulp(got, ref)
        assert m == 0.0, (cdf, n, w, S[w], K[w], T[w], got[w], ref[w])


@pytest.mark.parametrize("kind", ["all_small", "all_large", "edges", "mixed_chunks"])
def test_blackscholes_f32_regions_and_edges_bit_exact(gpu, oracle, kind):
    """The packed exact kernel evaluates both erfc regions and selects per lane: options whose
    arguments all fall in one region, special values (zeros, infinities, NaN, subnormals, huge
    and tiny times) and sizes that leave partial groups must still give the oracle's bits (two
    NaNs compare equal)."""
    rng = np.random.default_rng(17)
    if kind == "all_small":              # S ~ K and short T: |d| well below 2/3*sqrt(2)
        n = 3 * 2048 + 5
        S = rng.uniform(50, 51, n).astype(np.float32)
        K = (S * rng.uniform(0.999, 1.001, n)).astype(np.float32)
        T = rng.uniform(0.01, 0.02, n).astype(np.float32)
    elif kind == "all_large":            # deep in or out of the money: |d| > 3
        n = 2 * 2048 + 2
        S = rng.uniform(5, 6, n).astype(np.float32)
        K = rng.uniform(90, 100, n).astype(np.float32)
        T = rng.uniform(0.25, 0.5, n).astype(np.float32)
    elif kind == "edges":
        vals = np.array([0.0, -0.0, 1e-45, 1e-38, 1e-20, 0.5, 1.0, 2.0, 1e20, 3e38, np.inf, -np.inf, np.nan, -1.0],
                        np.float32)
        S, K, T = (a.ravel().astype(np.float32) for a in np.meshgrid(vals, vals, vals, indexing="ij"))
        n = S.size
    else:                                # the configuration's distribution, chunks partly filled
        n = 7 * 2048 + 1027
        S, K, T = bs_inputs(n, np.float32, seed=23)
    c, p = gpu.blackscholes(to_dev(S), to_dev(K), to_dev(T), 0.02, 0.30)
    rc, rp = oracle.bs(S, K, T, 0.02, 0.30)
    for got, ref in ((host(c), rc), (host(p), rp)):
        same = (got.view(np.uint32) == ref.view(np.uint32)) | (np.isnan(got) & np.isnan(ref))
        w = np.flatnonzero(~same)
        assert w.size == 0, (kind, w[:5], S[w[:5]], K[w[:5]], T[w[:5]], got[w[:5]], ref[w[:5]])


@pytest.mark.parametrize("n", [1, 3, 4099, 1 << 18])
def test_blackscholes_f64_bit_exact(gpu, oracle, n):
    S, K, T = bs_inputs(n, np.float64, seed=n + 7)
    c, p = gpu.blackscholes(to_dev(S), to_dev(K), to_dev(T), 0.02, 0.30)
    rc, rp = oracle.bs(S, K, T, 0.02, 0.30)
    assert oracle.max_ulp(host(c), rc)[0] == 0.0
    assert oracle.max_ulp(host(p), rp)[0] == 0.0


def test_blackscholes_f32_full_size_and_fp64_error(gpu, oracle):
    """2^24 options: bit-exact against the oracle; error against the FP64 evaluation reported."""
    n = 1 << 24
    S, K, T = bs_inputs(n, np.float32, seed=2024)
    c, p = gpu.blackscholes(to_dev(S), to_dev(K), to_dev(T), 0.02, 0.30)
    gc, gp = host(c), host(p)
    rc, rp = oracle.bs(S, K, T, 0.02, 0.30, threads=0)
    assert oracle.max_ulp(gc, rc)[0] == 0.0
    assert oracle.max_ulp(gp, rp)[0] == 0.0
    c64, p64 = oracle.bs(S.astype(np.float64), K.astype(np.float64), T.astype(np.float64), 0.02, 0.30)
    scale = np.maximum(np.abs(c64), 1.0)
    err = np.max(np.abs(gc - c64) / scale)
    assert err < 1e-4           # absolute error per unit of price, FP32 vs FP64 evaluation of the statement
    # put-call parity as a size-independent property
    parity = np.abs((gc.astype(np.float64) - gp) - (S - K * np.exp(-0.02 * T.astype(np.float64))))
    assert np.max(parity / (1 + K)) < 5e-5


def test_blackscholes_fused_within_bound(gpu, oracle):
    n = 1 << 18
    S, K, T = bs_inputs(n, np.float32, seed=3)
    c, p = gpu.blackscholes(to_dev(S), to_dev(K), to_dev(T), 0.02, 0.30, fused=True)
    rc, rp = oracle.bs(S, K, T, 0.02, 0.30)
    c64, _ = oracle.bs(S.astype(np.float64), K.astype(np.float64), T.astype(np.float64), 0.02, 0.30)
    # fused and unfused FP32 both within 1e-4 absolute of the FP64 evaluation (prices up to ~30)
    assert np.max(np.abs(host(c) - c64) / np.maximum(np.abs(c64), 1)) < 1e-4
    assert np.max(np.abs(rc - c64) / np.maximum(np.abs(c64), 1)) < 1e-4


@pytest.mark.parametrize("kind", ["config", "all_small", "all_large", "edges"])
def test_blackscholes_fused_packed_matches_one_lane(gpu, kind):
    """The fused mode's packed kernel (two options per instruction) gives the one-lane fused
    kernel's bits.  Misaligned tables take the one-lane kernel; the same options are priced
    through both."""
    rng = np.random.default_rng(29)
    if kind == "config":
        n = 5 * 2048 + 13
        S, K, T = bs_inputs(n, np.float32, seed=31)
    elif kind == "all_small":
        n = 2048 + 6
        S = rng.uniform(50, 51, n).astype(np.float32)
        K = (S * rng.uniform(0.999, 1.001, n)).astype(np.float32)
        T = rng.uniform(0.01, 0.02, n).astype(np.float32)
    elif kind == "all_large":
        n = 2048 + 7
        S = rng.uniform(5, 6, n).astype(np.float32)
        K = rng.uniform(90, 100, n).astype(np.float32)
        T = rng.uniform(0.25, 0.5, n).astype(np.float32)
    else:
        vals = np.array([0.0, -0.0, 1e-45, 1e-38, 0.5, 1.0, 2.0, 1e20, 3e38, np.inf, -np.inf, np.nan, -1.0],
                        np.float32)
        S, K, T = (a.ravel().astype(np.float32) for a in np.meshgrid(vals, vals, vals, indexing="ij"))
        n = S.size

    def misaligned(a):
        buf = torch.empty(a.size + 1, dtype=torch.float32, device="cuda")
        view = buf[1:]
        view.copy_(torch.from_numpy(a))
        return view

    c, p = gpu.blackscholes(to_dev(S), to_dev(K), to_dev(T), 0.02, 0.30, fused=True)
    oc = torch.empty(n + 1, dtype=torch.float32, device="cuda")[1:]
    op = torch.empty(n + 1, dtype=torch.float32, device="cuda")[1:]
    c1, p1 = gpu.blackscholes(misaligned(S), misaligned(K), misaligned(T), 0.02, 0.30, call=oc, put=op, fused=True)
    for got, ref in ((host(c), host(c1)), (host(p), host(p1))):
        same = (got.view(np.uint32) == ref.view(np.uint32)) | (np.isnan(got) & np.isnan(ref))
        w = np.flatnonzero(~same)
        assert w.size == 0, (kind, w[:5], S[w[:5]], K[w[:5]], T[w[:5]], got[w[:5]], ref[w[:5]])


def ulp_dist_f32(a, b):
    """|a - b| in float32 ulps (ordered-integer distance); NaN against NaN is 0."""
    ia = a.view(np.int32).astype(np.int64)
    ib = b.view(np.int32).astype(np.int64)
    ia = np.where(ia < 0, -(ia & 0x7FFFFFFF), ia)
    ib = np.where(ib < 0, -(ib & 0x7FFFFFFF), ib)
    d = np.abs(ia - ib)
    return np.where(np.isnan(a) & np.isnan(b), 0, np.where(np.isnan(a) ^ np.isnan(b), 1 << 40, d))


def bs_terms64(oracle, S, K, T, r=0.02, v=0.30):
    """FP64 sizes of the two terms each price is the difference of (S N(d1), K e^-rT N(d2) for the
    call; K e^-rT N(-d2), S N(-d1) for the put), through NT2's FP64 normcdf."""
    S64, K64, T64 = (a.astype(np.float64) for a in (S, K, T))
    vda = v * np.sqrt(T64)
    d1 = (np.log(S64 / K64) + (r + 0.5 * v * v) * T64) / vda
    d2 = d1 - vda
    e = K64 * np.exp(-r * T64)
    N = lambda x: oracle.map_("normcdf", np.ascontiguousarray(x))
    return S64 * N(d1) + e * N(d2), e * N(-d2) + S64 * N(-d1)


# precision="fast": maximum errors over every option of the sample.  Against FP64 (normcdf
# form): |fast - fp64| <= FAST_EPS_OF_TERMS * 2^-24 * (the two terms' FP64 sizes) + FLT_MIN;
# NT2's exact FP32 arithmetic itself needs up to ~200 there.  Against the exact FP32 oracle:
# every price >= 0.01 within FAST_ULP ulps.
FAST_EPS_OF_TERMS = 384
FAST_ULP = 768
EXACT_EPS_OF_TERMS = 256


@pytest.mark.parametrize("cdf", ["normcdf", "fastnormcdf"])
def test_blackscholes_fast_mode_bounds(gpu, oracle, cdf):
    n = 1 << 21
    S, K, T = bs_inputs(n, np.float32, seed=91)
    c, p = gpu.blackscholes(to_dev(S), to_dev(K), to_dev(T), 0.02, 0.30, cdf=cdf, precision="fast")
    gc, gp = host(c), host(p)
    kind = 0 if cdf == "normcdf" else 1
    rc, rp = oracle.bs(S, K, T, 0.02, 0.30, cdf=kind)
    for got, ref32 in ((gc, rc), (gp, rp)):
        big = ref32 >= 0.01
        u = ulp_dist_f32(got[big], ref32[big])
        assert u.max() <= FAST_ULP, u.max()
        assert np.max(np.abs(got.astype(np.float64) - ref32) / np.maximum(1.0, np.abs(ref32))) <= 2e-5
    if kind == 0:
        c64, p64 = oracle.bs(S.astype(np.float64), K.astype(np.float64), T.astype(np.float64), 0.02, 0.30)
        tc, tp = bs_terms64(oracle, S, K, T)
        eps, tiny = 2.0 ** -24, 2.0 ** -126
        for got, ref32, ref64, terms in ((gc, rc, c64, tc), (gp, rp, p64, tp)):
            fast = np.abs(got.astype(np.float64) - ref64) / (eps * terms + tiny)
            exact = np.abs(ref32.astype(np.float64) - ref64) / (eps * terms + tiny)
            assert fast.max() <= FAST_EPS_OF_TERMS, fast.max()
            assert exact.max() <= EXACT_EPS_OF_TERMS, exact.max()


def test_blackscholes_demo_bit_exact(gpu, oracle):
    n = 100003
    rng = np.random.default_rng(11)
    S = rng.uniform(5, 30, n).astype(np.float32)
    X = rng.uniform(1, 100, n).astype(np.float32)
    T = rng.uniform(0.25, 10, n).astype(np.float32)
    r = rng.uniform(0.0, 0.05, n).astype(np.float32)
    v = rng.uniform(0.1, 0.5, n).astype(np.float32)
    R = host(gpu.blackscholes_demo(*(to_dev(a) for a in (S, X, T, r, v))))
    ref = oracle.bs_demo(S, X, T, r, v)
    m, w = oracle.max_ulp(R, ref)
    assert m == 0.0, (w, R[w], ref[w])


def _demo_tables(kind, rng):
    if kind == "edges":
        vals = np.array([0.0, -0.0, 1e-45, 1e-38, 0.5, 1.0, 2.0, 1e20, 3e38, np.inf, -np.inf, np.nan, -1.0],
                        np.float32)
        S, X, T = (a.ravel() for a in np.meshgrid(vals, vals, vals, indexing="ij"))
        n = S.size
        r = np.resize(np.array([0.02, 0.0, -0.5, np.inf, np.nan], np.float32), n)
        v = np.resize(np.array([0.3, 0.0, 1e-20, 5.0, -0.3, np.nan, np.inf], np.float32), n)
        return [np.ascontiguousarray(a, dtype=np.float32) for a in (S, X, T, r, v)]
    n = {"tail": 4 * 999 + 3, "config": 3 * 2048 + 1}[kind]
    return [rng.uniform(lo, hi, n).astype(np.float32)
            for lo, hi in ((5, 30), (1, 100), (0.25, 10), (0.0, 0.05), (0.1, 0.5))]


@pytest.mark.parametrize("kind", ["tail", "config", "edges"])
def test_blackscholes_demo_single_pass_and_generic_path_bit_exact(gpu, oracle, kind):
    """Aligned tables take one pass with the demo's local tables da, d1, d2 in registers;
    misaligned views take the generic two-statement lowering.  Both give the oracle's bits
    (two NaNs compare equal), including in place (R the same table as S), and the fused
    modes of the two paths agree bit for bit."""
    tabs = _demo_tables(kind, np.random.default_rng(5))
    n = tabs[0].size
    ref = oracle.bs_demo(*tabs)

    def check(got):
        same = (got.view(np.uint32) == ref.view(np.uint32)) | (np.isnan(got) & np.isnan(ref))
        w = np.flatnonzero(~same)
        assert w.size == 0, (kind, w[:5], [t[w[:5]] for t in tabs], got[w[:5]], ref[w[:5]])

    def misaligned(a):
        view = torch.empty(a.size + 1, dtype=torch.float32, device="cuda")[1:]
        view.copy_(torch.from_numpy(a))
        return view

    check(host(gpu.blackscholes_demo(*(to_dev(a) for a in tabs))))
    dev = [to_dev(a) for a in tabs]
    check(host(gpu.blackscholes_demo(*dev, out=dev[0])))           # R = S
    mis = [misaligned(a) for a in tabs]
    out = torch.empty(n + 1, dtype=torch.float32, device="cuda")[1:]
    check(host(gpu.blackscholes_demo(*mis, out=out)))
    f1 = host(gpu.blackscholes_demo(*(to_dev(a) for a in tabs), fused=True))
    f2 = host(gpu.blackscholes_demo(*mis, out=out, fused=True))
    same = (f1.view(np.uint32) == f2.view(np.uint32)) | (np.isnan(f1) & np.isnan(f2))
    assert same.all(), (kind, np.flatnonzero(~same)[:5])


def test_blackscholes_host_entry(gpu, oracle):
    n = (1 << 21) * 3 + 17   # several pipeline chunks and a ragged tail
    S, K, T = bs_inputs(n, np.float32, seed=77)
    ts = [torch.from_numpy(a).pin_memory() for a in (S, K, T)]
    call = torch.empty(n, dtype=torch.float32).pin_memory()
    put = torch.empty(n, dtype=torch.float32).pin_memory()
    gpu.blackscholes_host(*ts, 0.02, 0.30, call, put)
    rc, rp = oracle.bs(S, K, T, 0.02, 0.30)
    assert oracle.max_ulp(call.numpy(), rc)[0] == 0.0
    assert oracle.max_ulp(put.numpy(), rp)[0] == 0.0


def test_alias_rules(gpu):
    import nt2_gb300
    x = torch.ones(1024, device="cuda")
    # y aliases x with an offset: partial overlap is rejected
    with pytest.raises(nt2_gb300.NT2CudaError):
        gpu.saxpy(2.0, x[1:513], x[0:512])
    # exact aliasing Y = a*Y + Y is allowed and elementwise
    y = torch.full((1000,), 3.0, device="cuda")
    gpu.saxpy(2.0, y, y)
    assert torch.all(y == 9.0)


def test_autotune_and_tuning_roundtrip(gpu, oracle):
    u, w, ms = gpu.autotune("bs_f32", 1 << 20)
    assert u in (1, 2, 4) and w in (1, 2, 4, 8) and ms > 0
    text = gpu.tuning_export()
    assert "bs_f32@20" in text
    assert gpu.tuning_import(text) >= 1
    S, K, T = bs_inputs(1 << 20, np.float32, seed=1)
    c, p = gpu.blackscholes(to_dev(S), to_dev(K), to_dev(T), 0.02, 0.30)
    rc, _ = oracle.bs(S, K, T, 0.02, 0.30)
    assert oracle.max_ulp(host(c), rc)[0] == 0.0
