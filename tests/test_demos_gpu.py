"""NT2's demo programs, written as NT2 user code against the nt2cuda table front
end (nt2_gb300/demo/demos.cu), produce the oracle's results bit for bit."""
import os
import subprocess
import sys

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def demos(gpu):
    sys.path.insert(0, os.path.join(ROOT, "nt2_gb300", "demo"))
    import build_demos
    return build_demos.build()


def run(demos, tmp_path, cmd, n, arrays, outs, extra=()):
    files = []
    for i, a in enumerate(arrays):
        p = tmp_path / f"in{i}.bin"
        np.ascontiguousarray(a).tofile(p)
        files.append(str(p))
    out_files = [str(tmp_path / f"out{i}.bin") for i in range(outs)]
    r = subprocess.run([demos, cmd, str(n), *extra, *files, *out_files], capture_output=True, text=True,
                       timeout=300)
    assert r.returncode == 0, r.stderr
    return r.stdout, out_files


def test_saxpy_demo(demos, oracle, tmp_path):
    n = 100003
    rng = np.random.default_rng(1)
    x = rng.uniform(-1, 1, n).astype(np.float32)
    y = rng.uniform(-1, 1, n).astype(np.float32)
    _, (o,) = run(demos, tmp_path, "saxpy", n, [x, y], 1)
    ref = y.copy()
    oracle.load().nt2o_saxpy_f(2.5, x, ref, n, 1)
    assert np.array_equal(np.fromfile(o, np.float32).view(np.uint32), ref.view(np.uint32))


def test_sdot_demo(demos, oracle, tmp_path):
    n = 1 << 20
    rng = np.random.default_rng(2)
    x = rng.standard_normal(n).astype(np.float32)
    y = rng.standard_normal(n).astype(np.float32)
    out, _ = run(demos, tmp_path, "sdot", n, [x, y], 0)
    ref, ab = oracle.dot_fp64(x, y)
    assert abs(float(out) - ref) <= 2 ** -22 * ab


@pytest.mark.parametrize("form", ["bs", "bs_merged"])
def test_blackscholes_demo(demos, oracle, tmp_path, form):
    n = 50001
    rng = np.random.default_rng(3)
    S = rng.uniform(5, 30, n).astype(np.float32)
    X = rng.uniform(1, 100, n).astype(np.float32)
    T = rng.uniform(0.25, 10, n).astype(np.float32)
    r = rng.uniform(0, 0.05, n).astype(np.float32)
    v = rng.uniform(0.1, 0.5, n).astype(np.float32)
    _, (o,) = run(demos, tmp_path, form, n, [S, X, T, r, v], 1)
    ref = oracle.bs_demo(S, X, T, r, v)
    m, w = oracle.max_ulp(np.fromfile(o, np.float32), ref)
    assert m == 0.0, (form, w)


def test_rgb2grey_demo(demos, oracle, tmp_path):
    n = 640 * 480
    rng = np.random.default_rng(4)
    r, g, b = (rng.uniform(0, 255, n).astype(np.float32) for _ in range(3))
    _, (o,) = run(demos, tmp_path, "rgb2grey", n, [r, g, b], 1)
    ref = np.empty_like(r)
    oracle.load().nt2o_rgb2grey_f(r, g, b, ref, n, 1)
    assert np.array_equal(np.fromfile(o, np.float32).view(np.uint32), ref.view(np.uint32))


def test_rgb2grey_u8_demo(demos, oracle, tmp_path):
    n = 640 * 480 + 5
    rng = np.random.default_rng(6)
    r, g, b = (rng.integers(0, 256, n, dtype=np.uint8) for _ in range(3))
    _, (o,) = run(demos, tmp_path, "rgb2grey_u8", n, [r, g, b], 1)
    ref = np.empty_like(r)
    oracle.load().nt2o_rgb2grey_u8(r, g, b, ref, n, 1)
    assert np.array_equal(np.fromfile(o, np.uint8), ref)


def test_rgb2yuv_demo(demos, oracle, tmp_path):
    n = 128 * 128 + 3
    rng = np.random.default_rng(7)
    r, g, b = (rng.uniform(0, 255, n).astype(np.float32) for _ in range(3))
    _, outs = run(demos, tmp_path, "rgb2yuv", n, [r, g, b], 3)
    for o, ref in zip(outs, oracle.rgb2yuv(r, g, b)):
        assert np.array_equal(np.fromfile(o, np.float32).view(np.uint32), ref.view(np.uint32))


def test_sigmadelta_demo(demos, oracle, tmp_path):
    npix, nf = 333 * 97, 6
    rng = np.random.default_rng(5)
    bg = rng.integers(16, 240, npix)
    frames = np.concatenate([np.clip(bg + rng.integers(-8, 9, npix), 0, 255) for _ in range(nf)]).astype(np.uint8)
    frames[3 * npix + 100:3 * npix + 400] = 255
    _, (ob, ov, ol) = run(demos, tmp_path, "sigmadelta", npix, [frames], 3, extra=(str(nf),))
    rb, rv, rl = oracle.sigmadelta(frames, npix, npix, nf, init=True)
    assert np.array_equal(np.fromfile(ob, np.uint8), rb)
    assert np.array_equal(np.fromfile(ov, np.uint8), rv)
    assert np.array_equal(np.fromfile(ol, np.uint8), rl[(nf - 2) * npix:])    # the demo keeps the last label


def test_stats_demo(demos, gpu, tmp_path):
    """NT2-spelled reductions and cumulative functions give the C-ABI results bit for bit."""
    import torch
    rows, cols = 1000, 37
    rng = np.random.default_rng(9)
    A = (rng.standard_normal(rows * cols) * 2 + 1).astype(np.float32)
    _, outs = run(demos, tmp_path, "stats", rows, [A], 7, extra=(str(cols),))
    got = [np.fromfile(o, np.float32) for o in outs]
    Ad = torch.from_numpy(A).cuda()
    h = lambda t: (torch.cuda.synchronize(), t.cpu().numpy())[1]
    expect = [h(gpu.reduce("mean", Ad, rows, cols, 1)), h(gpu.reduce("var", Ad, rows, cols, 2)),
              h(gpu.reduce("max", Ad, rows, cols, 1)), h(gpu.reduce("asum1", Ad, rows, cols, 2)),
              h(gpu.cumulative("cumsum", Ad, rows, cols, 1)), h(gpu.cumulative("cumsum", Ad, rows, cols, 2))]
    for g, e in zip(got[:6], expect):
        assert np.array_equal(g.view(np.uint32), e.view(np.uint32))
    gl = [h(gpu.reduce(op, Ad, rows, cols, 0))[0] for op in ("sum", "norm2", "max", "stdev")]
    assert np.array_equal(got[6].view(np.uint32), np.array(gl, np.float32).view(np.uint32))


def test_trig_demo(demos, oracle, tmp_path):
    """Trigonometric functors inside an NT2 statement (each node reduces its element on its own,
    NT2's scalar code) and under a fold: the statement is bit-exact, the fold within its FP64 bound."""
    n = 100003
    x = np.random.default_rng(12).uniform(-60, 60, n).astype(np.float32)
    _, (oy, og) = run(demos, tmp_path, "trig", n, [x], 2)
    s = oracle.trig("sin", x)
    c = oracle.trig("cos", x)
    t = oracle.trig("tan", x * np.float32(0.25))
    cp = oracle.trig("cospi", x)
    sp = oracle.trig("sinpi", x)
    want = (s + c * t) + cp * sp
    got = np.fromfile(oy, np.float32)
    assert np.array_equal(got.view(np.uint32), want.view(np.uint32))
    g = float(np.fromfile(og, np.float32)[0])
    ref = float(np.sum(s.astype(np.float64)))
    assert abs(g - ref) <= 4 * 2.0 ** -24 * float(np.sum(np.abs(s.astype(np.float64)))), (g, ref)


def test_pow_demo(demos, oracle, tmp_path):
    """nt2::pow of two tables and of a table with a scalar exponent inside one statement, and
    cbrt + logspace_add: bit-exact against NT2's SIMD forms."""
    n = 50021
    rng = np.random.default_rng(13)
    x = (rng.uniform(-1, 1, n) * np.exp(rng.uniform(-8, 8, n))).astype(np.float32)
    y = rng.uniform(-12, 12, n).astype(np.float32)
    y[::3] = np.round(y[::3])                      # integer exponents: negative bases stay real
    _, (oz, ow) = run(demos, tmp_path, "pow", n, [x, y], 2)
    want = oracle.pow_(x, y) + oracle.pow_(y, np.full(n, 2.0, np.float32))
    got = np.fromfile(oz, np.float32)
    bad = ~(np.isnan(got) & np.isnan(want)) & (got.view(np.uint32) != want.view(np.uint32))
    assert not bad.any(), (np.flatnonzero(bad)[:5], x[bad][:5], y[bad][:5], got[bad][:5], want[bad][:5])
    want = oracle.map_("cbrt", x) + oracle.map2("logspace_add", x, y)
    got = np.fromfile(ow, np.float32)
    bad = ~(np.isnan(got) & np.isnan(want)) & (got.view(np.uint32) != want.view(np.uint32))
    assert not bad.any(), (np.flatnonzero(bad)[:5], x[bad][:5], y[bad][:5])


def test_trigx_demo(demos, oracle, tmp_path):
    """Composed trigonometric functors through the C++ front end: csc(x) + asind(x*1e-3f) + secpi(x)
    in one statement, bit-exact against NT2's compositions."""
    n = 30011
    x = np.random.default_rng(14).uniform(-600, 600, n).astype(np.float32)
    x[::7] = np.round(x[::7] * 2) / 2              # integers and halves: secpi's NaNs
    _, (oy, ow) = run(demos, tmp_path, "trigx", n, [x], 2)
    want = (oracle.trigx("csc", x) + oracle.trigx("asind", x * np.float32(1e-3))) + oracle.trigx("secpi", x)
    got = np.fromfile(oy, np.float32)
    bad = ~(np.isnan(got) & np.isnan(want)) & (got.view(np.uint32) != want.view(np.uint32))
    assert not bad.any(), (np.flatnonzero(bad)[:5], x[bad][:5], got[bad][:5], want[bad][:5])
    want = (oracle.trig("cot", x) + oracle.trig("sind", x)) + oracle.trig("tanpi", x * np.float32(0.01))
    got = np.fromfile(ow, np.float32)
    bad = ~(np.isnan(got) & np.isnan(want)) & (got.view(np.uint32) != want.view(np.uint32))
    assert not bad.any(), (np.flatnonzero(bad)[:5], x[bad][:5], got[bad][:5], want[bad][:5])


def test_io_demo(demos, tmp_path):
    """nt2cuda::load reads a table file written from Python, the statement runs on the device, and
    nt2cuda::save writes the result back with its extent."""
    from nt2_gb300 import tableio
    rows, cols = 37, 1000
    A = np.random.default_rng(4).standard_normal(rows * cols)
    src, dst = tmp_path / "a.tbl", tmp_path / "b.tbl"
    tableio.save(src, A, rows, cols)
    r = subprocess.run([demos, "io", "0", str(src), str(dst)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    assert r.stdout.split() == [str(rows), str(cols)]
    B, ext = tableio.load(dst)
    assert ext == (rows, cols)
    assert np.array_equal(B, A * 2.0 + 1.0)


def test_reshape_demo(demos, tmp_path):
    """B = expr takes the right-hand side's extent (NT2's run_assign resizes the lhs):
    same element count in another shape, then another element count."""
    rows, cols = 37, 11
    A = np.arange(rows * cols, dtype=np.float32) * 0.5 - 3
    f = tmp_path / "A"
    A.tofile(f)
    outs = [tmp_path / f"B{k}" for k in (1, 2, 3)]
    r = subprocess.run([demos, "reshape", str(rows), str(cols), str(f), *map(str, outs)], capture_output=True,
                       text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    lines = dict((l.split()[0], l.split()[1:]) for l in r.stdout.splitlines())
    assert lines["B1"] == [str(rows), str(cols)]
    assert lines["B2"] == [str(cols), str(rows)]
    assert lines["B3"] == ["5", "7"]
    assert np.array_equal(np.fromfile(outs[0], np.float32), A * np.float32(2) + np.float32(1))
    assert np.array_equal(np.fromfile(outs[1], np.float32), A + np.float32(1))
    C = np.arange(1, 36, dtype=np.float32)
    assert np.array_equal(np.fromfile(outs[2], np.float32), C * np.float32(3))
    assert float(lines["G"][0]) == float(C.sum())
    assert float(lines["G"][1]) == float((C.astype(np.float64) ** 2).sum())
