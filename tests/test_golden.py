"""Committed golden vectors (tests/golden/nt2_golden.npz, made by
tests/golden/make_golden.py on x86-64): the oracle rebuilt on this machine
and the CUDA path must both reproduce them bit for bit (NaNs compare equal)."""
import os

import numpy as np
import pytest
import torch

G = np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "nt2_golden.npz"))


def same(a, b):
    a = np.asarray(a)
    b = np.asarray(b)
    if a.dtype.kind == "f":
        both_nan = np.isnan(a) & np.isnan(b)
        return bool(np.all((a.view(np.uint8).reshape(a.shape + (-1,)) == b.view(np.uint8).reshape(b.shape + (-1,)))
                           .all(axis=-1) | both_nan))
    return bool(np.array_equal(a, b))


OPS32 = ["exp", "log", "erfc", "normcdf", "fastnormcdf", "sqrt", "exp2", "exp10", "log2", "log10", "expm1", "log1p"]
OPS64 = ["exp", "log", "erfc", "normcdf", "sqrt", "exp2", "exp10", "log2", "log10", "expm1", "log1p"]


@pytest.mark.parametrize("op", OPS32)
def test_oracle_reproduces_golden_f32(oracle, op):
    assert same(oracle.map_(op, G[f"map_f32_{op}_x"]), G[f"map_f32_{op}_y"])


@pytest.mark.parametrize("op", OPS64)
def test_oracle_reproduces_golden_f64(oracle, op):
    assert same(oracle.map_(op, G[f"map_f64_{op}_x"]), G[f"map_f64_{op}_y"])


def test_oracle_reproduces_golden_statements(oracle):
    for tag in ("f32", "f64"):
        c, p = oracle.bs(G[f"bs_{tag}_S"], G[f"bs_{tag}_K"], G[f"bs_{tag}_T"], 0.02, 0.30, cdf=0)
        assert same(c, G[f"bs_{tag}_call"]) and same(p, G[f"bs_{tag}_put"])
    c, p = oracle.bs(G["bs_f32_S"], G["bs_f32_K"], G["bs_f32_T"], 0.02, 0.30, cdf=1)
    assert same(c, G["bs_f32_fast_call"]) and same(p, G["bs_f32_fast_put"])
    assert same(oracle.bs_demo(G["demo_S"], G["demo_X"], G["demo_T"], G["demo_r"], G["demo_v"]), G["demo_R"])
    npix, nf = int(G["sd_npix"]), int(G["sd_nframes"])
    b, v, lab = oracle.sigmadelta(G["sd_frames"], npix, npix, nf, init=True)
    assert same(b, G["sd_bkg"]) and same(v, G["sd_var"]) and same(lab, G["sd_labels"])


def dev(a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def host(t):
    torch.cuda.synchronize()
    return t.cpu().numpy()


@pytest.mark.gpu
@pytest.mark.parametrize("op", OPS32)
def test_device_reproduces_golden_f32(gpu, op):
    assert same(host(gpu.map_(op, dev(G[f"map_f32_{op}_x"]))), G[f"map_f32_{op}_y"])


@pytest.mark.gpu
@pytest.mark.parametrize("op", OPS64)
def test_device_reproduces_golden_f64(gpu, op):
    assert same(host(gpu.map_(op, dev(G[f"map_f64_{op}_x"]))), G[f"map_f64_{op}_y"])


@pytest.mark.gpu
def test_device_reproduces_golden_statements(gpu):
    for tag in ("f32", "f64"):
        c, p = gpu.blackscholes(dev(G[f"bs_{tag}_S"]), dev(G[f"bs_{tag}_K"]), dev(G[f"bs_{tag}_T"]), 0.02, 0.30)
        assert same(host(c), G[f"bs_{tag}_call"]) and same(host(p), G[f"bs_{tag}_put"])
    c, p = gpu.blackscholes(dev(G["bs_f32_S"]), dev(G["bs_f32_K"]), dev(G["bs_f32_T"]), 0.02, 0.30, cdf="fastnormcdf")
    assert same(host(c), G["bs_f32_fast_call"]) and same(host(p), G["bs_f32_fast_put"])
    R = gpu.blackscholes_demo(*(dev(G[k]) for k in ("demo_S", "demo_X", "demo_T", "demo_r", "demo_v")))
    assert same(host(R), G["demo_R"])
    y = dev(G["saxpy_y"])
    gpu.saxpy(2.5, dev(G["saxpy_x"]), y)
    assert same(host(y), G["saxpy_out"])
    from nt2_gb300 import video  # noqa: F401
    npix, nf = int(G["sd_npix"]), int(G["sd_nframes"])
    e = {"frames": dev(G["sd_frames"]), "frame_stride": npix, "width": 64, "height": 48,
         "bkg": torch.zeros(npix, dtype=torch.uint8, device="cuda"),
         "var": torch.zeros(npix, dtype=torch.uint8, device="cuda"),
         "labels": torch.zeros(nf * npix, dtype=torch.uint8, device="cuda"), "label_stride": npix}
    gpu.sigmadelta_batch([e], nf, init=True)
    assert same(host(e["bkg"]), G["sd_bkg"]) and same(host(e["var"]), G["sd_var"])
    assert same(host(e["labels"])[: (nf - 1) * npix], G["sd_labels"])


def test_oracle_reproduces_golden_images(oracle):
    gr = np.empty_like(G["grey8_r"])
    oracle.load().nt2o_rgb2grey_u8(G["grey8_r"], G["grey8_g"], G["grey8_b"], gr, gr.size, 1)
    assert same(gr, G["grey8_out"])
    for got, key in zip(oracle.rgb2yuv(G["yuv_r"], G["yuv_g"], G["yuv_b"]), ("yuv_y", "yuv_u", "yuv_v")):
        assert same(got, G[key])
    for pack in (1, 8):
        assert same(oracle.mandelbrot_grid(-1.5, 1.5, -1.5, 1.5, 160, 160, pack=pack), G[f"mandel_p{pack}"])


@pytest.mark.gpu
def test_gpu_reproduces_golden_images(gpu):
    import torch
    d = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()
    h = lambda t: (torch.cuda.synchronize(), t.cpu().numpy())[1]
    assert same(h(gpu.rgb2grey(d(G["grey8_r"]), d(G["grey8_g"]), d(G["grey8_b"]))), G["grey8_out"])
    for got, key in zip(gpu.rgb2yuv(d(G["yuv_r"]), d(G["yuv_g"]), d(G["yuv_b"])), ("yuv_y", "yuv_u", "yuv_v")):
        assert same(h(got), G[key])
    for pack in (1, 8):
        assert same(h(gpu.mandelbrot_grid(-1.5, 1.5, -1.5, 1.5, 160, 160, pack=pack)), G[f"mandel_p{pack}"])
