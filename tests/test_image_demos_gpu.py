"""rgb2grey over uint8 planes, rgb2yuv and mandelbrot on the GPU against the CPU oracle.

All three are bit-exact with unfused arithmetic: the uint8 grey levels and
the int32 escape counts are integer results, and rgb2yuv's float planes
must equal NT2's three passes bit for bit.  With fused = 1 (hardware FMA)
rgb2yuv's y plane is held to 2 ulpdist (bounds for u, v in the test) and
the uint8 grey level to +-1.
"""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def to_dev(a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def host(t):
    torch.cuda.synchronize()
    return t.cpu().numpy()


SIZES = [0, 1, 15, 16, 17, 33, 1000, 4097, 1920 * 1080 + 7]


@pytest.mark.parametrize("n", SIZES)
def test_rgb2grey_u8_bit_exact(gpu, oracle, n):
    rng = np.random.default_rng(n + 3)
    r, g, b = (rng.integers(0, 256, n, dtype=np.uint8) for _ in range(3))
    if n >= 4:
        r[:4] = g[:4] = b[:4] = np.array([0, 255, 1, 254], np.uint8)
    out = host(gpu.rgb2grey(to_dev(r), to_dev(g), to_dev(b)))
    ref = np.empty_like(r)
    oracle.load().nt2o_rgb2grey_u8(r, g, b, ref, n, 1)
    assert np.array_equal(out, ref)


def test_rgb2grey_u8_every_grey_level(gpu, oracle):
    """All 2^24 (r, g, b) triples: bit-exact against the oracle."""
    v = np.arange(1 << 24, dtype=np.uint32)
    r, g, b = ((v >> s) & 255 for s in (0, 8, 16))
    r, g, b = (x.astype(np.uint8) for x in (r, g, b))
    out = host(gpu.rgb2grey(to_dev(r), to_dev(g), to_dev(b)))
    ref = np.empty_like(r)
    oracle.load().nt2o_rgb2grey_u8(r, g, b, ref, r.size, 0)
    assert np.array_equal(out, ref)
    fused = host(gpu.rgb2grey(to_dev(r), to_dev(g), to_dev(b), fused=True))
    assert np.abs(fused.astype(np.int16) - ref.astype(np.int16)).max() <= 1


def test_rgb2grey_u8_misaligned_views(gpu, oracle):
    n = 5000
    rng = np.random.default_rng(5)
    base = [to_dev(rng.integers(0, 256, n + 3, dtype=np.uint8)) for _ in range(3)]
    views = [t[1:n + 1] for t in base]
    out = torch.empty(n + 5, dtype=torch.uint8, device="cuda")[3:n + 3]
    gpu.rgb2grey(*views, out=out)
    r, g, b = (host(v) for v in views)
    ref = np.empty(n, np.uint8)
    oracle.load().nt2o_rgb2grey_u8(r, g, b, ref, n, 1)
    assert np.array_equal(host(out), ref)


@pytest.mark.parametrize("n", SIZES)
def test_rgb2yuv_bit_exact(gpu, oracle, n):
    rng = np.random.default_rng(n + 11)
    r, g, b = (rng.uniform(0, 255, n).astype(np.float32) for _ in range(3))
    dy, du, dv = (host(t) for t in gpu.rgb2yuv(to_dev(r), to_dev(g), to_dev(b)))
    y, u, v = oracle.rgb2yuv(r, g, b, threads=1)
    for got, ref in ((dy, y), (du, u), (dv, v)):
        assert np.array_equal(got.view(np.uint32), ref.view(np.uint32))


def test_rgb2yuv_fused_bounds(gpu, oracle):
    n = 1 << 20
    rng = np.random.default_rng(2)
    r, g, b = (rng.uniform(0, 255, n).astype(np.float32) for _ in range(3))
    got = [host(t) for t in gpu.rgb2yuv(to_dev(r), to_dev(g), to_dev(b), fused=True)]
    ref = oracle.rgb2yuv(r, g, b)
    # y (three positive terms, two roundings saved) within 2 in NT2's ulpdist (adjacent floats
    # are 0.5 apart).  u = c*(b - y) and v = c*(r - y) have no fma of their own: they differ only
    # through y, by at most c*(|dy| + one spacing of the difference) + one spacing of the product.
    assert oracle.max_ulp(got[0], ref[0])[0] <= 2.0
    dy = np.abs(got[0].astype(np.float64) - ref[0])
    for k, c, x in ((1, 0.492, b), (2, 0.877, r)):
        diff = np.abs(x - ref[0])
        lim = c * (dy + 2 * np.spacing(diff)) + 2 * np.spacing(np.abs(ref[k]))
        assert np.all(np.abs(got[k].astype(np.float64) - ref[k]) <= lim)


def test_rgb2yuv_rejects_overlap(gpu, cuda_lib):
    t = torch.zeros(4096, dtype=torch.float32, device="cuda")
    r, g, b = (torch.zeros(1000, dtype=torch.float32, device="cuda") for _ in range(3))
    st = cuda_lib.nt2cuda_rgb2yuv_f32(r.data_ptr(), g.data_ptr(), b.data_ptr(), t.data_ptr(),
                                      t.data_ptr() + 400, t.data_ptr() + 8000, 1000, 0,
                                      torch.cuda.current_stream().cuda_stream)
    assert st == 8  # NT2CUDA_ERR_ALIAS
    st = cuda_lib.nt2cuda_rgb2yuv_f32(r.data_ptr(), g.data_ptr(), b.data_ptr(), r.data_ptr(),
                                      t.data_ptr(), t.data_ptr() + 8000, 1000, 0,
                                      torch.cuda.current_stream().cuda_stream)
    assert st == 8


@pytest.mark.parametrize("pack", [1, 2, 4, 8, 16, 32])
@pytest.mark.parametrize("hw", [(1, 1), (7, 5), (100, 100), (203, 97)])
def test_mandelbrot_grid_bit_exact(gpu, oracle, pack, hw):
    h, w = hw
    got = host(gpu.mandelbrot_grid(-1.5, 1.5, -1.5, 1.5, h, w, pack=pack))
    ref = oracle.mandelbrot_grid(-1.5, 1.5, -1.5, 1.5, h, w, pack=pack)
    assert np.array_equal(got, ref)


def test_mandelbrot_demo_size(gpu, oracle):
    """The demo's largest size, 1600 x 1600 over [-1.5, 1.5]^2, AVX pack width."""
    got = host(gpu.mandelbrot_grid(-1.5, 1.5, -1.5, 1.5, 1600, 1600, pack=8))
    ref = oracle.mandelbrot_grid(-1.5, 1.5, -1.5, 1.5, 1600, 1600, pack=8)
    assert np.array_equal(got, ref)
    assert got.max() == 256 and got.min() >= 1


@pytest.mark.parametrize("pack", [1, 8])
def test_mandelbrot_tables_match_grid(gpu, oracle, pack):
    """arrayfun over explicit A, B tables (the demo's expand_to(linspace) materialised)."""
    h = w = 321
    la, lb = oracle.linspace(-2.0, 1.0, w), oracle.linspace(-1.25, 1.25, h)
    A = np.repeat(la, h).astype(np.float32)           # A(i,j) = la[j], column-major
    B = np.tile(lb, w).astype(np.float32)             # B(i,j) = lb[i]
    got = host(gpu.mandelbrot(to_dev(A), to_dev(B), pack=pack))
    assert np.array_equal(got, oracle.mandelbrot(A, B, pack=pack))
    assert np.array_equal(got, host(gpu.mandelbrot_grid(-2.0, 1.0, -1.25, 1.25, h, w, pack=pack)))


def test_mandelbrot_pack_semantics(gpu, oracle):
    """Points whose orbit leaves the disc and comes back: the count depends on the pack."""
    rng = np.random.default_rng(4)
    n = 1 << 16
    A = rng.uniform(-2.2, 2.2, n).astype(np.float32)
    B = rng.uniform(-2.2, 2.2, n).astype(np.float32)
    outs = {}
    for pack in (1, 8, 32):
        outs[pack] = host(gpu.mandelbrot(to_dev(A), to_dev(B), pack=pack))
        assert np.array_equal(outs[pack], oracle.mandelbrot(A, B, pack=pack))
    # a lane of a wider pack runs at least the trips it runs alone, so its count can only grow
    assert np.all(outs[8] >= outs[1]) and np.all(outs[32] >= outs[8])


def test_mandelbrot_bad_args(gpu, cuda_lib):
    A = torch.zeros(10, dtype=torch.float32, device="cuda")
    C = torch.zeros(10, dtype=torch.int32, device="cuda")
    s = torch.cuda.current_stream().cuda_stream
    assert cuda_lib.nt2cuda_mandelbrot_f32(A.data_ptr(), A.data_ptr(), C.data_ptr(), 10, 3, s) == 1
    assert cuda_lib.nt2cuda_mandelbrot_f32(A.data_ptr(), A.data_ptr(), A.data_ptr(), 10, 8, s) == 8
    assert cuda_lib.nt2cuda_mandelbrot_grid_f32(0.0, 1.0, 0.0, 1.0, 0, 5, None, 8, s) == 0
