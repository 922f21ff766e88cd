"""Guard bands: no entry point writes outside its output tables.

compute-sanitizer is not available here, so every output table is the middle of
a larger buffer whose two 1024-element margins hold a sentinel pattern; after
the call the margins must be unchanged, bit for bit.  Sizes are odd (vector
tails), and each case also runs on a view shifted by one element (the
misaligned path of every kernel).
"""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

G = 1024
SENT = {torch.float32: (torch.int32, 0x7FBADBAD), torch.float64: (torch.int64, 0x7FF4DEADBEEF0001),
        torch.uint8: (torch.uint8, 0xA5), torch.int32: (torch.int32, 0x7FBADBAD)}
SIZES = [1, 3, 4097, 65537]


class Guarded:
    """A table of n elements between two sentinel margins (shifted by `shift` elements)."""

    def __init__(self, n, dtype, shift=0):
        self.n, self.shift, self.dtype = n, shift, dtype
        self.buf = torch.empty(n + 2 * G + shift, dtype=dtype, device="cuda")
        it, pat = SENT[dtype]
        self.buf.view(it).fill_(pat)
        self.view = self.buf[G + shift:G + shift + n]

    def intact(self):
        it, pat = SENT[self.dtype]
        bits = self.buf.view(it)
        lo = bits[:G + self.shift]
        hi = bits[G + self.shift + self.n:]
        return bool((lo == pat).all()) and bool((hi == pat).all())


def rand(n, dtype, lo=-2.0, hi=2.0, seed=0):
    g = torch.Generator(device="cuda").manual_seed(seed)
    return (torch.rand(n, generator=g, device="cuda", dtype=dtype) * (hi - lo) + lo)


def sync():
    torch.cuda.synchronize()


@pytest.mark.parametrize("dtype", [torch.float32, torch.float64])
@pytest.mark.parametrize("shift", [0, 1])
def test_map_outputs(gpu, dtype, shift):
    for op in gpu.OPS:
        if op == "fastnormcdf" and dtype == torch.float64:
            continue
        for n in SIZES:
            x = rand(n, dtype, 0.1 if op.startswith("log") or op == "sqrt" else -2.0, 2.0, n)
            for simd in ((False, True) if op in ("sin", "cos", "tan", "sinpi", "cospi") else (False,)):
                for fused in (False, True):
                    out = Guarded(n, dtype, shift)
                    gpu.map_(op, x, out=out.view, fused=fused, simd128=simd)
                    sync()
                    assert out.intact(), (op, n, shift, simd, fused)


@pytest.mark.parametrize("shift", [0, 1])
def test_elementwise_statements(gpu, cuda_lib, shift):
    for n in SIZES:
        x = rand(n, torch.float32, seed=1)
        y = Guarded(n, torch.float32, shift)
        y.view.copy_(rand(n, torch.float32, seed=2))
        gpu.saxpy(2.5, x, y.view)
        S, K, T = rand(n, torch.float32, 5, 30, 3), rand(n, torch.float32, 1, 100, 4), rand(n, torch.float32, 0.25, 10, 5)
        for prec in ("exact", "fused", "fast"):
            call, put = Guarded(n, torch.float32, shift), Guarded(n, torch.float32, shift)
            gpu.blackscholes(S, K, T, 0.02, 0.3, call.view, put.view, precision=prec)
            sync()
            assert call.intact() and put.intact(), (n, prec)
        r, g, b = (rand(n, torch.float32, 0, 255, 6 + k) for k in range(3))
        gr = Guarded(n, torch.float32, shift)
        gpu.rgb2grey(r, g, b, out=gr.view)
        r8, g8, b8 = (t.to(torch.uint8) for t in (r, g, b))
        gr8 = Guarded(n, torch.uint8, shift)
        gpu.rgb2grey(r8, g8, b8, out=gr8.view)
        yy, uu, vv = (Guarded(n, torch.float32, shift) for _ in range(3))
        st = cuda_lib.nt2cuda_rgb2yuv_f32(r.data_ptr(), g.data_ptr(), b.data_ptr(), yy.view.data_ptr(),
                                          uu.view.data_ptr(), vv.view.data_ptr(), n, 0,
                                          torch.cuda.current_stream().cuda_stream)
        assert st == 0
        at = Guarded(n, torch.float32, shift)
        gpu.atan2(x, r, out=at.view)
        pw = Guarded(n, torch.float32, shift)
        gpu.pow(r, x, out=pw.view)
        m2 = []
        for op in gpu.OPS2:
            m2.append(Guarded(n, torch.float32, shift))
            gpu.map2(op, r, x, out=m2[-1].view)
        cm = Guarded(n, torch.int32, shift)
        gpu.mandelbrot(rand(n, torch.float32, -1.5, 1.5, 9), rand(n, torch.float32, -1.5, 1.5, 10), out=cm.view)
        sync()
        for t in (y, gr, gr8, yy, uu, vv, at, pw, cm, *m2):
            assert t.intact(), n
    h, w = 37, 41
    grid = Guarded(h * w, torch.int32, shift)
    gpu.mandelbrot_grid(-1.5, 1.5, -1.5, 1.5, h, w, out=grid.view)
    sync()
    assert grid.intact()


@pytest.mark.parametrize("dtype", [torch.float32, torch.float64])
@pytest.mark.parametrize("shape", [(1, 1), (33, 7), (4097, 3), (70000, 2), (5, 9000)])
def test_reduction_and_scan_outputs(gpu, dtype, shape):
    rows, cols = shape
    A = rand(rows * cols, dtype, 0.5, 1.5, rows + cols)
    for shift in (0, 1):
        for op in ("sum", "asum1", "asum2", "norm2", "mean", "var", "stdev", "max", "min", "prod",
                   "all", "any", "none"):
            for dim in (0, 1, 2):
                m = 1 if dim == 0 else (cols if dim == 1 else rows)
                odt = torch.uint8 if op in ("all", "any", "none") else dtype
                out = Guarded(m, odt, shift)
                gpu.reduce(op, A, rows, cols, dim, out=out.view)
                sync()
                assert out.intact(), (op, dim, shift)
        for op in ("cumsum", "cumprod", "cummax", "cummin"):
            for dim in (1, 2):
                out = Guarded(rows * cols, dtype, shift)
                gpu.cumulative(op, A, rows, cols, dim, out=out.view)
                sync()
                assert out.intact(), (op, dim, shift)
        for fn in (lambda o: gpu.globalsum(A, out=o), lambda o: gpu.dot(A, A, out=o)):
            out = Guarded(1, dtype, shift)
            fn(out.view)
            sync()
            assert out.intact()


def test_sigmadelta_outputs(gpu):
    nframes = 5
    entries, guards = [], []
    for k, (w, h) in enumerate([(17, 3), (64, 16), (333, 7)]):
        npix = w * h
        frames = torch.randint(0, 256, (nframes * npix,), dtype=torch.uint8, device="cuda")
        bkg, var = Guarded(npix, torch.uint8, k % 2), Guarded(npix, torch.uint8, k % 2)
        labels = Guarded((nframes - 1) * npix, torch.uint8, k % 2)
        entries.append({"frames": frames, "frame_stride": npix, "bkg": bkg.view, "var": var.view,
                        "labels": labels.view, "label_stride": npix, "width": w, "height": h})
        guards += [bkg, var, labels]
    gpu.sigmadelta_batch(entries, nframes, init=True)
    sync()
    assert all(g.intact() for g in guards)
