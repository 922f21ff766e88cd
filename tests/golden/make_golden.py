"""Generate tests/golden/nt2_golden.npz: seeded inputs and the oracle's outputs
for the elementwise statements, Black-Scholes, and sigmadelta.

The oracle restates NT2's algorithms (oracle/nt2_oracle.c); NT2 itself needs
Boost and cannot be built here.  The fixture pins those results across
machines: the oracle rebuilt on another architecture, and the GPU path, must
reproduce it bit for bit (tests/test_golden.py).

    python tests/golden/make_golden.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))
import oracle_lib  # noqa: E402

SPECIALS = [0.0, -0.0, 1.0, -1.0, 0.5, 2.0, np.inf, -np.inf, np.nan, 88.5, -88.5, 1e-40, -3.0, 709.0, -708.0]


def inputs(op, n, dtype, seed):
    rng = np.random.default_rng(seed)
    lo, hi = {"exp": (-100, 100), "log": (0, 100), "sqrt": (0, 100), "exp2": (-150, 150), "exp10": (-45, 45),
              "log2": (0, 100), "log10": (0, 100), "expm1": (-100, 100), "log1p": (-1, 100)}.get(op, (-10, 10))
    x = rng.uniform(lo, hi, n).astype(dtype)
    sp = np.array(SPECIALS, dtype)
    x[: len(sp)] = sp
    return x


def main():
    out = {}
    for i, op in enumerate(["exp", "log", "erfc", "normcdf", "fastnormcdf", "sqrt", "exp2", "exp10", "log2", "log10",
                            "expm1", "log1p"]):
        x = inputs(op, 2048, np.float32, 100 + i)
        out[f"map_f32_{op}_x"] = x
        out[f"map_f32_{op}_y"] = oracle_lib.map_(op, x)
    for i, op in enumerate(["exp", "log", "erfc", "normcdf", "sqrt", "exp2", "exp10", "log2", "log10", "expm1",
                            "log1p"]):
        x = inputs(op, 2048, np.float64, 200 + i)
        out[f"map_f64_{op}_x"] = x
        out[f"map_f64_{op}_y"] = oracle_lib.map_(op, x)
    rng = np.random.default_rng(7)
    n = 4099
    for dt, tag in ((np.float32, "f32"), (np.float64, "f64")):
        S = rng.uniform(5, 30, n).astype(dt)
        K = rng.uniform(1, 100, n).astype(dt)
        T = rng.uniform(0.25, 10, n).astype(dt)
        out[f"bs_{tag}_S"], out[f"bs_{tag}_K"], out[f"bs_{tag}_T"] = S, K, T
        c, p = oracle_lib.bs(S, K, T, 0.02, 0.30, cdf=0)
        out[f"bs_{tag}_call"], out[f"bs_{tag}_put"] = c, p
        if dt == np.float32:
            c, p = oracle_lib.bs(S, K, T, 0.02, 0.30, cdf=1)
            out["bs_f32_fast_call"], out["bs_f32_fast_put"] = c, p
    S, X, T = (rng.uniform(a, b, n).astype(np.float32) for a, b in ((5, 30), (1, 100), (0.25, 10)))
    r = rng.uniform(0, 0.05, n).astype(np.float32)
    v = rng.uniform(0.1, 0.5, n).astype(np.float32)
    out.update(demo_S=S, demo_X=X, demo_T=T, demo_r=r, demo_v=v, demo_R=oracle_lib.bs_demo(S, X, T, r, v))
    x = rng.uniform(-1, 1, n).astype(np.float32)
    y = rng.uniform(-1, 1, n).astype(np.float32)
    yy = y.copy()
    oracle_lib.load().nt2o_saxpy_f(2.5, x, yy, n, 1)
    out.update(saxpy_x=x, saxpy_y=y, saxpy_out=yy)
    npix, nf = 64 * 48, 6
    bg = rng.integers(16, 240, npix)
    frames = np.concatenate([np.clip(bg + rng.integers(-8, 9, npix), 0, 255) for _ in range(nf)]).astype(np.uint8)
    frames[2 * npix + 100:2 * npix + 700] = 255
    b, vv, lab = oracle_lib.sigmadelta(frames, npix, npix, nf, init=True)
    out.update(sd_frames=frames, sd_bkg=b, sd_var=vv, sd_labels=lab, sd_npix=np.array(npix), sd_nframes=np.array(nf))
    # image statements: uint8 rgb2grey, rgb2yuv, and the mandelbrot program at pack widths 1 and 8
    r8, g8, b8 = (rng.integers(0, 256, 5000, dtype=np.uint8) for _ in range(3))
    gr8 = np.empty_like(r8)
    oracle_lib.load().nt2o_rgb2grey_u8(r8, g8, b8, gr8, r8.size, 1)
    out.update(grey8_r=r8, grey8_g=g8, grey8_b=b8, grey8_out=gr8)
    rf, gf, bf = (rng.uniform(0, 255, 5000).astype(np.float32) for _ in range(3))
    yy_, uu_, vv_ = oracle_lib.rgb2yuv(rf, gf, bf)
    out.update(yuv_r=rf, yuv_g=gf, yuv_b=bf, yuv_y=yy_, yuv_u=uu_, yuv_v=vv_)
    for pack in (1, 8):
        out[f"mandel_p{pack}"] = oracle_lib.mandelbrot_grid(-1.5, 1.5, -1.5, 1.5, 160, 160, pack=pack)
    np.savez_compressed(os.path.join(HERE, "nt2_golden.npz"), **out)
    print("wrote", os.path.join(HERE, "nt2_golden.npz"), sum(a.nbytes for a in out.values()), "bytes raw")


if __name__ == "__main__":
    main()
