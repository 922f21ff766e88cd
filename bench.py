#!/usr/bin/env python3
"""Benchmark: FP32 Black-Scholes call+put over 2^24 options on one GB300 per rank.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference] [--suite]

One step is one evaluation of the Black-Scholes statement over the whole
2^24-option batch (S, K, T resident in HBM; 335 MB of compulsory traffic,
larger than the 129 MB L2, so no flush is needed between steps).  Prints one
JSON line.  --suite also prints one line per other configuration (saxpy,
sdot, inner/outer folds, FP64 Black-Scholes, batched sigma-delta).
--impl reference times the CPU restatement of NT2's SIMD+OpenMP path on the
host cores instead (rank 0 only).
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "Black-Scholes options/s & % HBM peak; serving p99 latency vs launch-per-call"
N_OPTIONS = 1 << 24
R, SIGMA = 0.02, 0.30
BYTES_PER_OPTION = 20            # S, K, T read; call, put written (float32)
NOMINAL_HBM_GBS = 8000.0
INFLIGHT = 3                     # launches in flight, for both launching serving modes
MODES = ("resident", "batched", "launch_per_request")


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def profiled_traffic(name: str):
    """dram bytes per launch recorded from an ncu capture in profiles/<name>.md ("traffic_bytes_per_launch: X")."""
    p = os.path.join(ROOT, "profiles", name + ".md")
    try:
        for line in open(p):
            if line.strip().startswith("traffic_bytes_per_launch:"):
                return float(line.split(":", 1)[1].strip().split()[0])
    except Exception:
        pass
    return None


DATA = ("synthetic (seeded counter-based uniforms: S~U[5,30], K~U[1,100], T~U[0.25,10]; r=0.02, sigma=0.30)")


def headline_config(n: int, ws: int) -> dict:
    return {"workload": "Black-Scholes call+put, FP32, 2^24 options per GPU, normcdf via erfc, "
                        "NT2 unfused arithmetic (bit-exact with the oracle)",
            "options_per_gpu": n, "parallelism": f"replicas x{ws}",
            "l2": "inputs+outputs 335 MB > 129 MB L2, no flush needed"}


# ------------------------------------------------------------------ clocks
class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled while the bench runs."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.samples = []
        self.proc = None
        self.thread = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "100"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except Exception:
            self.proc = None
            return self
        self.thread = threading.Thread(target=self._read, daemon=True)
        self.thread.start()
        return self

    def _read(self):
        for line in self.proc.stdout:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                self.samples.append((time.time(), float(parts[1]), float(parts[2]), parts[5:9]))
            except ValueError:
                pass

    def stop(self):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self, t0: float, t1: float):
        win = [s for s in self.samples if t0 - 0.15 <= s[0] <= t1 + 0.15]
        src = "timed_region"
        if not win:
            win = self.samples
            src = "whole_run"
        if not win:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"], "samples": 0}
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for s in win for i, v in enumerate(s[3]) if v.lower() == "active"})
        return {"sm_mhz": statistics.median(s[1] for s in win), "sm_max_mhz": max(s[2] for s in win),
                "reasons": reasons, "samples": len(win), "window": src}


# --------------------------------------------------------------- helpers
def dist_env():
    from nt2_gb300 import replicas
    return replicas.env()


def max_over_ranks(x: float, ws: int):
    from nt2_gb300 import replicas
    return replicas.max_over_ranks(x, ws)


def barrier(ws: int):
    from nt2_gb300 import replicas
    replicas.barrier(ws)


def bs_tables(n: int, seed: int):
    import torch
    import nt2_gb300.api as api
    S = torch.empty(n, dtype=torch.float32, device="cuda")
    K = torch.empty(n, dtype=torch.float32, device="cuda")
    T = torch.empty(n, dtype=torch.float32, device="cuda")
    api.fill_uniform(S, 5.0, 30.0, seed * 3 + 1)
    api.fill_uniform(K, 1.0, 100.0, seed * 3 + 2)
    api.fill_uniform(T, 0.25, 10.0, seed * 3 + 3)
    return S, K, T


def time_device(fn, steps: int, warmup: int, ws: int):
    """CUDA-event time of `steps` calls on torch's current stream, max over ranks (ms per step)."""
    import torch
    for _ in range(warmup):
        fn()
    torch.cuda.synchronize()
    barrier(ws)
    torch.cuda.synchronize()
    stream = torch.cuda.current_stream()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    t0 = time.time()
    e0.record(stream)
    for _ in range(steps):
        fn()
    e1.record(stream)
    torch.cuda.synchronize()
    t1 = time.time()
    barrier(ws)
    ms = e0.elapsed_time(e1) / steps
    return max_over_ranks(ms, ws), t0, t1


# ---------------------------------------------------------- CPU baseline
def _oracle():
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    import oracle_lib
    return oracle_lib


def cpu_rate(fn, units: float, seconds: float = 2.0, min_reps: int = 5):
    """Median units/s of fn() after one warm-up call, over >= min_reps calls and about `seconds`."""
    fn()
    rates = []
    t_end = time.perf_counter() + seconds
    while time.perf_counter() < t_end or len(rates) < min_reps:
        t = time.perf_counter()
        fn()
        rates.append(units / (time.perf_counter() - t))
    return statistics.median(rates), len(rates)


def nt2_threading(L, n: int, elem_size: int) -> dict:
    """How NT2's transform spawner treats a table of n elements on this host: grain = L2 bytes /
    sizeof(T), OpenMP only when n > 8 * grain (shared_memory/transform.hpp:38-48)."""
    l2 = int(L.nt2o_l2_bytes())
    grain = max(1, l2 // elem_size)
    par = n > 8 * grain
    return {"l2_bytes": l2, "grain": grain, "parallel": par, "threads": int(L.nt2o_max_threads()) if par else 1}


def cpu_baseline(S, K, T, seconds: float = 3.0):
    """The oracle's NT2-restated Black-Scholes on the host cores over the same 2^24-option batch
    (options/s, median of reps): the scalar+OpenMP build NT2 runs on aarch64 is the baseline; the
    compiler-vectorised build of the same loops is reported beside it as an upper bound."""
    import numpy as np
    oracle_lib = _oracle()
    n = S.size
    call = np.empty_like(S)
    put = np.empty_like(S)

    def rate(variant):
        L = oracle_lib.load(variant)
        v, reps = cpu_rate(lambda: L.nt2o_bs_f(S, K, T, R, SIGMA, call, put, n, 0, 0), n, seconds)
        return v, reps, L

    value, reps, L = rate("libnt2oracle.so")
    vec, vreps, _ = rate("libnt2oracle_vec.so")
    th = nt2_threading(L, n, 4)
    return {"value": value, "unit": "options/s", "cores": th["threads"], "kind": "port",
            "sample": f"the full {n}-option batch (the GPU's inputs), {reps} reps, median; NT2 scalar+OpenMP "
                      f"restatement (oracle/nt2_oracle.c, -O2), NT2's spawner rule: grain {th['grain']} "
                      f"elements (L2 {th['l2_bytes']} B), parallel={th['parallel']}",
            "vectorised_upper_bound": {"value": vec, "unit": "options/s", "reps": vreps,
                                       "build": "same loops, -O3 auto-vectorised"}}


# ------------------------------------------------------------- accuracy
def _ulp_dist_f32(a, b):
    """|a - b| in units in the last place of float32 (ordered-integer distance; NaN-aware)."""
    import numpy as np
    ia = a.view(np.int32).astype(np.int64)
    ib = b.view(np.int32).astype(np.int64)
    ia = np.where(ia < 0, -(ia & 0x7FFFFFFF), ia)
    ib = np.where(ib < 0, -(ib & 0x7FFFFFFF), ib)
    d = np.abs(ia - ib)
    both_nan = np.isnan(a) & np.isnan(b)
    one_nan = np.isnan(a) ^ np.isnan(b)
    d = np.where(both_nan, 0, d)
    return np.where(one_nan, np.int64(1) << 40, d)


def normcdf64(x):
    try:
        from scipy.special import ndtr
        return ndtr(x)
    except Exception:                                   # the NT2 FP64 normcdf of the oracle
        import numpy as np
        o = _oracle()
        out = np.empty_like(x)
        o.load().nt2o_map_d(o.OP["normcdf"], np.ascontiguousarray(x), out, x.size)
        return out


class BSReference:
    """FP32 oracle and FP64 reference prices of one batch, for the error of each result."""

    def __init__(self, S, K, T):
        import numpy as np
        o = _oracle()
        L = o.load()
        n = S.size
        self.rc = np.empty(n, np.float32)
        self.rp = np.empty(n, np.float32)
        L.nt2o_bs_f(S, K, T, R, SIGMA, self.rc, self.rp, n, 0, 0)
        S64, K64, T64 = (a.astype(np.float64) for a in (S, K, T))
        self.dc = np.empty(n)
        self.dp = np.empty(n)
        L.nt2o_bs_d(S64, K64, T64, R, SIGMA, self.dc, self.dp, n, 0)
        # the sizes of the two terms each price is the difference of: an error relative to them
        # is what FP32 can promise where the price cancels
        vda = SIGMA * np.sqrt(T64)
        d1 = (np.log(S64 / K64) + (R + 0.5 * SIGMA * SIGMA) * T64) / vda
        d2 = d1 - vda
        e = K64 * np.exp(-R * T64)
        self.scale_c = S64 * normcdf64(d1) + e * normcdf64(d2)
        self.scale_p = e * normcdf64(-d2) + S64 * normcdf64(-d1)

    def errors(self, call, put, floor: float = 0.01) -> dict:
        import numpy as np
        eps = 2.0 ** -24
        out = {}
        u_or = max(int(_ulp_dist_f32(call, self.rc).max()), int(_ulp_dist_f32(put, self.rp).max()))
        out["max_ulp_vs_oracle"] = u_or
        ec = np.abs(call.astype(np.float64) - self.dc)
        ep = np.abs(put.astype(np.float64) - self.dp)
        out["max_abs_err_vs_fp64"] = float(max(ec.max(), ep.max()))
        # eps = 2^-24 of the larger term, or of FLT_MIN where the terms are below the normal range
        tiny = 2.0 ** -126
        out["max_err_vs_fp64_in_eps_of_terms"] = float(max((ec / (eps * self.scale_c + tiny)).max(),
                                                           (ep / (eps * self.scale_p + tiny)).max()))
        c64 = self.dc.astype(np.float32)
        p64 = self.dp.astype(np.float32)
        mc = self.dc >= floor
        mp = self.dp >= floor
        out[f"max_ulp_vs_fp64_prices_ge_{floor}"] = int(max(_ulp_dist_f32(call[mc], c64[mc]).max(initial=0),
                                                           _ulp_dist_f32(put[mp], p64[mp]).max(initial=0)))
        mo_c = self.rc >= floor
        mo_p = self.rp >= floor
        out[f"max_ulp_vs_oracle_prices_ge_{floor}"] = int(max(_ulp_dist_f32(call[mo_c], self.rc[mo_c]).max(initial=0),
                                                             _ulp_dist_f32(put[mo_p], self.rp[mo_p]).max(initial=0)))
        return out


# ------------------------------------------- the other configurations
def _roof(bytes_, ms, peak):
    gbs = bytes_ / (ms * 1e-3) / 1e9
    return {"bound": "hbm", "achieved": gbs, "peak": peak, "unit": "GB/s", "frac": gbs / peak,
            "algorithmic_bytes_per_launch": int(bytes_)}


def _cpu(value, unit, cores, sample, reps):
    return {"value": value, "unit": unit, "cores": cores, "kind": "port", "reps": reps, "sample": sample}


def config_lines(ws: int, steps: int, warmup: int) -> dict:
    """Every other configuration of the benchmark list, measured the same way as the headline:
    device time with inputs resident (rotating copies larger than L2 where one table fits in it),
    the fraction of the measured copy bandwidth, the NT2-restated CPU path timed on the same
    inputs on the host cores, and each result's error against the oracle and an FP64 oracle."""
    import numpy as np
    import torch
    import nt2_gb300.api as api
    from nt2_gb300 import video
    o = _oracle()
    L = o.load()
    peak, _ = peaks()
    eps = 2.0 ** -24
    out = {}
    K = lambda d: max(3, min(steps, d))

    def guarded(name, fn):
        try:
            out[name] = fn()
        except Exception as e:                     # one configuration's failure is reported, not fatal
            out[name] = {"error": repr(e)[:300]}
        torch.cuda.empty_cache()

    def saxpy():
        n = 1 << 24
        xs = [torch.empty(n, device="cuda") for _ in range(4)]
        ys = [torch.empty(n, device="cuda") for _ in range(4)]
        for i in range(4):
            api.fill_uniform(xs[i], -1, 1, 1 + i)
            api.fill_uniform(ys[i], -1, 1, 11 + i)
        x0, y0 = xs[0].cpu().numpy(), ys[0].cpu().numpy()
        api.autotune("saxpy_f32", n)
        it = [0]

        def step():
            i = it[0] & 3
            it[0] += 1
            api.saxpy(2.5, xs[i], ys[i])
        ms, _, _ = time_device(step, K(200), warmup, ws)
        # accuracy on fresh copies of pair 0
        xg = torch.from_numpy(x0).cuda()
        yg = torch.from_numpy(y0.copy()).cuda()
        api.saxpy(2.5, xg, yg)
        got = yg.cpu().numpy()
        ref = y0.copy()
        L.nt2o_saxpy_f(2.5, x0, ref, n, 0)
        r64 = 2.5 * x0.astype(np.float64) + y0.astype(np.float64)
        yc = y0.copy()
        rate, reps = cpu_rate(lambda: L.nt2o_saxpy_f(2.5, x0, yc, n, 0), n)
        th = nt2_threading(L, n, 4)
        return {"ms": ms, "value": ws * n / (ms * 1e-3), "unit": "elements/s", "roofline": _roof(12 * n, ms, peak),
                "l2": "4 rotating (x, y) pairs, 536 MB > L2",
                "cpu_baseline": _cpu(rate, "elements/s", th["threads"], f"same 2^24-element x, y; NT2 spawner "
                                     f"parallel={th['parallel']}", reps),
                "error": {"mismatches_vs_oracle": int(np.count_nonzero(got.view(np.uint32) != ref.view(np.uint32))),
                          "max_ulp_vs_fp64": int(_ulp_dist_f32(got, r64.astype(np.float32)).max())}}

    def sdot():
        n = 1 << 26
        x = torch.empty(n, device="cuda")
        y = torch.empty(n, device="cuda")
        api.fill_normal(x, 1)
        api.fill_normal(y, 2)
        xh, yh = x.cpu().numpy(), y.cpu().numpy()
        ref, ab = o.dot_fp64(xh, yh)
        res = {}
        oc = torch.empty(1, device="cuda")
        cpu_v, reps = cpu_rate(lambda: L.nt2o_dot_omp_f(xh, yh.ctypes.data, n, 8, 0), n)
        cpu_err = abs(float(L.nt2o_dot_omp_f(xh, yh.ctypes.data, n, 8, 0)) - ref) / (eps * ab)
        for comp in (True, False):
            ms, _, _ = time_device(lambda: api.dot(x, y, compensated=comp, out=oc), K(100), warmup, ws)
            g = float(api.dot(x, y, compensated=comp).cpu()[0])
            res["compensated" if comp else "plain"] = {
                "ms": ms, "value": ws * n / (ms * 1e-3), "unit": "elements/s", "roofline": _roof(8 * n, ms, peak),
                "error": {"abs_err_vs_fp64": abs(g - ref), "err_in_eps_sum_abs": abs(g - ref) / (eps * ab)}}
        res["cpu_baseline"] = _cpu(cpu_v, "elements/s", int(L.nt2o_max_threads()),
                                   "same 2^26 x, y; NT2's OpenMP fold (static chunks, partials summed)", reps)
        res["cpu_baseline"]["err_in_eps_sum_abs"] = cpu_err
        res["l2"] = "inputs 536 MB > L2"
        return res

    def folds():
        rows, cols = 8192, 4096
        As = [torch.empty(rows * cols, device="cuda") for _ in range(4)]
        for i in range(4):
            api.fill_normal(As[i], 3 + i)
        Ah = As[0].cpu().numpy()
        o32c, o64c, abc = o.inner_fold(Ah, rows, cols, lanes=4)
        o32r, o64r, abr = o.outer_fold(Ah, rows, cols)
        res = {}
        for dim, name, m, ref64, ab, cpu32 in ((1, "column_sums_inner_fold", cols, o64c, abc, o32c),
                                               (2, "row_sums_outer_fold", rows, o64r, abr, o32r)):
            oo = torch.empty(m, device="cuda")
            it = [0]

            def step(dim=dim, oo=oo):
                i = it[0] & 3
                it[0] += 1
                api.sum_colmajor(As[i], rows, cols, dim, out=oo)
            ms, _, _ = time_device(step, K(100), warmup, ws)
            g = api.sum_colmajor(As[0], rows, cols, dim).cpu().numpy().astype(np.float64)
            if dim == 1:
                tmp = np.empty(cols, np.float32)
                fn = lambda: L.nt2o_inner_fold_f(Ah, rows, cols, 4, tmp.ctypes.data, None, None, 0)
                how = "NT2's inner_fold: columns over the threads, 4-lane fold per column"
            else:
                tmp = np.empty(rows, np.float32)
                fn = lambda: L.nt2o_outer_fold_nt2_f(Ah, rows, cols, tmp, 0)
                how = "NT2's in-cache outer_fold: 16-row chunks over the threads, columns added in turn"
            rate, reps = cpu_rate(fn, rows * cols)
            res[name] = {
                "ms": ms, "value": ws * rows * cols / (ms * 1e-3), "unit": "elements/s",
                "roofline": _roof(4 * rows * cols + 4 * m, ms, peak),
                "cpu_baseline": _cpu(rate, "elements/s", int(L.nt2o_max_threads()), f"same 8192x4096 table; {how}",
                                     reps),
                "error": {"max_err_in_eps_sum_abs": float((np.abs(g - ref64) / (eps * ab)).max()),
                          "cpu_nt2_fp32_max_err_in_eps_sum_abs":
                              float((np.abs(cpu32.astype(np.float64) - ref64) / (eps * ab)).max())}}
        res["l2"] = "4 rotating 134 MB tables, 536 MB > L2"
        return res

    def bs_f64():
        n = 1 << 24
        Sd = torch.empty(n, dtype=torch.float64, device="cuda")
        Kd = torch.empty(n, dtype=torch.float64, device="cuda")
        Td = torch.empty(n, dtype=torch.float64, device="cuda")
        api.fill_uniform(Sd, 5, 30, 1)
        api.fill_uniform(Kd, 1, 100, 2)
        api.fill_uniform(Td, 0.25, 10, 3)
        c = torch.empty_like(Sd)
        p = torch.empty_like(Sd)
        ms, _, _ = time_device(lambda: api.blackscholes(Sd, Kd, Td, R, SIGMA, call=c, put=p), K(20), warmup, ws)
        api.blackscholes(Sd, Kd, Td, R, SIGMA, call=c, put=p)
        Sh, Kh, Th = (a.cpu().numpy() for a in (Sd, Kd, Td))
        rc, rp = np.empty(n), np.empty(n)
        L.nt2o_bs_d(Sh, Kh, Th, R, SIGMA, rc, rp, n, 0)
        gc, gp = c.cpu().numpy(), p.cpu().numpy()
        mism = int(np.count_nonzero(gc.view(np.uint64) != rc.view(np.uint64)) +
                   np.count_nonzero(gp.view(np.uint64) != rp.view(np.uint64)))
        rate, reps = cpu_rate(lambda: L.nt2o_bs_d(Sh, Kh, Th, R, SIGMA, rc, rp, n, 0), n)
        th = nt2_threading(L, n, 8)
        return {"ms": ms, "value": ws * n / (ms * 1e-3), "unit": "options/s",
                "roofline": _roof(40 * n, ms, peak), "bound_note": "FP64 issue (GB300's FP64 rate), not HBM",
                "cpu_baseline": _cpu(rate, "options/s", th["threads"], "same 2^24 FP64 options; NT2 double path",
                                     reps),
                "error": {"mismatches_vs_fp64_oracle": mism,
                          "note": "the FP64 oracle is NT2's double arithmetic restated; 0 = bit-exact"}}

    def bs_demo():
        # the demo's own statement (demo/blackscholes/nt2/blackandscholes_nt2.cpp:55-59): five input
        # tables, one output, one fused transform; r ~ U[0.01, 0.05] and v ~ U[0.1, 0.5] per option
        n = 1 << 24
        tabs = [torch.empty(n, device="cuda") for _ in range(5)]
        for t, (lo, hi), sd in zip(tabs, ((5.0, 30.0), (1.0, 100.0), (0.25, 10.0), (0.01, 0.05), (0.1, 0.5)),
                                   (21, 22, 23, 24, 25)):
            api.fill_uniform(t, lo, hi, sd)
        res = torch.empty(n, device="cuda")
        ms, _, _ = time_device(lambda: api.blackscholes_demo(*tabs, out=res), K(50), warmup, ws)
        api.blackscholes_demo(*tabs, out=res)
        hs = [t.cpu().numpy() for t in tabs]
        ref = np.empty(n, np.float32)
        L.nt2o_bs_demo_f(*hs, ref, n, 0)
        got = res.cpu().numpy()
        mism = int(np.count_nonzero(got.view(np.uint32) != ref.view(np.uint32)))
        rate, reps = cpu_rate(lambda: L.nt2o_bs_demo_f(*hs, ref, n, 0), n)
        th = nt2_threading(L, n, 4)
        return {"ms": ms, "value": ws * n / (ms * 1e-3), "unit": "options/s",
                "roofline": _roof(24 * n, ms, peak),
                "inputs": "S ~ U[5,30], X ~ U[1,100], T ~ U[0.25,10], r ~ U[0.01,0.05], v ~ U[0.1,0.5] tables",
                "cpu_baseline": _cpu(rate, "options/s", th["threads"],
                                     "same 2^24 options; the demo statement, NT2 scalar+OpenMP restated", reps),
                "error": {"mismatches_vs_oracle": mism, "note": "NT2's FP32 arithmetic restated; 0 = bit-exact"}}

    def sigmadelta():
        batch = video.make_batch(256, 8, seed=11)
        torch.cuda.synchronize()
        plan = api.SigmaDeltaPlan(batch, 8, init=True)
        ms, _, _ = time_device(plan.launch, K(20), warmup, ws)
        plan.close()
        torch.cuda.synchronize()
        frames = [e["frames"].cpu().numpy() for e in batch]
        npix = np.array([e["width"] * e["height"] for e in batch], np.uint64)
        fstride = np.array([e["frame_stride"] for e in batch], np.uint64)
        bk = [np.zeros(int(m), np.uint8) for m in npix]
        vr = [np.zeros(int(m), np.uint8) for m in npix]
        lb = [np.zeros(7 * int(m), np.uint8) for m in npix]
        keep = [(C.c_void_p * len(a))(*[x.ctypes.data for x in a]) for a in (frames, bk, vr, lb)]
        pf, pb, pv, pl = (C.cast(a, C.c_void_p) for a in keep)
        run = lambda: L.nt2o_sigmadelta_batch_u8(len(batch), pf, fstride.ctypes.data, npix.ctypes.data, 8, pb,
                                                 pv, pl, 1, 0)
        pfr = video.pixel_frames(batch, 8, True)
        rate, reps = cpu_rate(run, pfr, seconds=3.0, min_reps=3)
        mism = 0
        for e, b, v, l in zip(batch, bk, vr, lb):
            m = e["width"] * e["height"]
            mism += int(np.count_nonzero(e["bkg"].cpu().numpy() != b) + np.count_nonzero(e["var"].cpu().numpy() != v))
            gl = e["labels"].cpu().numpy()
            for f in range(7):
                lo = f * e["label_stride"]
                mism += int(np.count_nonzero(gl[lo:lo + m] != l[f * m:(f + 1) * m]))
        return {"ms": ms, "value": ws * pfr / (ms * 1e-3), "unit": "pixel-frames/s",
                "roofline": _roof(video.bytes_moved(batch, 8, True), ms, peak),
                "streams": len(batch), "pixels": int(npix.sum()), "launch": "one persistent kernel in a CUDA graph",
                "cpu_baseline": _cpu(rate, "pixel-frames/s", int(L.nt2o_max_threads()),
                                     "same 256 streams x 8 frames; each stream's NT2 statement on one thread "
                                     "(below NT2's spawner threshold), streams spread over the threads", reps),
                "error": {"mismatched_bytes_vs_oracle": mism}}

    guarded("saxpy_f32_2^24", saxpy)
    guarded("sdot_f32_2^26", sdot)
    guarded("folds_f32_8192x4096", folds)
    guarded("blackscholes_f64_2^24", bs_f64)
    guarded("blackscholes_demo_f32_2^24", bs_demo)
    guarded("sigmadelta_u8_256x8", sigmadelta)
    return out


# -------------------------------------------------------------- serving
def serving_bench(seconds: float = 1.0, rates=(1000, 5000, 10000, 20000, 50000), seed: int = 7):
    """Poisson arrivals of Black-Scholes requests (sizes log-uniform 256..2^22 options) into the
    server's three modes on the same GPU: a resident kernel draining a request ring, one launch
    per step over the admitted requests, and one launch per request (the last two allowed the
    same number of launches in flight).  The trace is replayed natively
    (nt2cuda_server_replay): arrivals, completion waits and releases run in C++ threads, so the
    numbers are the server's, not a Python client's."""
    import numpy as np
    import torch
    from nt2_gb300.server import Server
    pool_n = 1 << 24
    S, K, T = bs_tables(pool_n, seed=99)
    torch.cuda.synchronize()
    rng = np.random.default_rng(seed)
    sp, kp, tp = S.data_ptr(), K.data_ptr(), T.data_ptr()
    out = {}

    def replay(mode, sizes, offs, arrivals):
        srv = Server(budget_bytes=40 << 30, max_batch_requests=4096, max_inflight_batches=INFLIGHT,
                     mode={"resident": "resident", "batched": "batched", "launch_per_request": "launch"}[mode],
                     wait_timeout_ms=20000)
        lat, elapsed = srv.replay(sp, kp, tp, R, SIGMA, offs, sizes, arrivals)
        st = srv.stats()
        srv.close()
        lat_us = lat.astype(np.float64) / 1e3
        return {"requests": int(sizes.size), "options_per_s": float(sizes.sum() / elapsed),
                "p50_us": float(np.percentile(lat_us, 50)), "p99_us": float(np.percentile(lat_us, 99)),
                "launches": int(st["launches"]), "batches": int(st["batches"]),
                "admission_waits": int(st["admission_waits"]),
                "peak_reserved_gb": round(st["peak_reserved_bytes"] / 1e9, 2)}

    for rate in rates:
        nreq = max(8, int(rate * seconds))
        sizes = np.exp(rng.uniform(math.log(256), math.log(1 << 22), nreq)).astype(np.uint64)
        offs = ((rng.integers(0, pool_n - (1 << 22), nreq) // 4) * 4).astype(np.uint64)
        arrivals = (np.cumsum(rng.exponential(1.0 / rate, nreq)) * 1e9).astype(np.uint64)
        out[f"{rate}_req_s"] = {m: replay(m, sizes, offs, arrivals) for m in MODES}
    # saturation: every request offered at once (small requests, where launch cost dominates)
    sat_rng = np.random.default_rng(seed + 1)
    nreq, lo, hi = 20000, 256, 1 << 14
    sizes = np.exp(sat_rng.uniform(math.log(lo), math.log(hi), nreq)).astype(np.uint64)
    offs = ((sat_rng.integers(0, pool_n - hi, nreq) // 4) * 4).astype(np.uint64)
    zero = np.zeros(nreq, np.uint64)
    sat = {m: replay(m, sizes, offs, zero) for m in MODES}
    for m in ("resident", "batched"):
        sat[f"throughput_ratio_{m}"] = sat[m]["options_per_s"] / sat["launch_per_request"]["options_per_s"]
    out["saturation_small_requests"] = sat
    out["inflight_launches_both_modes"] = INFLIGHT
    return out


# ------------------------------------------------------------- our arm
def run_ours(args):
    import torch
    ws, rank, local = dist_env()
    if ws > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    else:
        torch.cuda.set_device(0)
    import nt2_gb300.api as api
    from nt2_gb300._lib import lib
    api.init(torch.cuda.current_device())
    L = lib()
    n = N_OPTIONS
    S, K, T = bs_tables(n, seed=rank)
    call = torch.empty_like(S)
    put = torch.empty_like(S)
    stream = torch.cuda.current_stream().cuda_stream
    sp, kp, tp, cp, pp = S.data_ptr(), K.data_ptr(), T.data_ptr(), call.data_ptr(), put.data_ptr()

    # the project's autotuner picks unroll and grid waves per precision mode (outside the timed region)
    tuned = {}
    for key in ("bs_f32", "bs_f32_fused", "bs_f32_fast"):
        u, w, tms = api.autotune(key, n)
        tuned[key] = {"unroll": u, "waves": w, "ms": tms}

    def make_step(prec):
        def step():
            st = L.nt2cuda_blackscholes_f32(sp, kp, tp, R, SIGMA, cp, pp, n, 0, prec, stream)
            if st:
                raise RuntimeError(f"blackscholes status {st}")
        return step

    step = make_step(0)
    sampler = ClockSampler(torch.cuda.current_device()).start()
    time.sleep(0.3)
    ms, t0, t1 = time_device(step, args.steps, max(args.warmup, 3), ws)
    modes = {}
    for name, prec in (("fused", 1), ("fast", 2)):
        mms, _, _ = time_device(make_step(prec), min(args.steps, 500), max(args.warmup, 3), ws)
        gbs = BYTES_PER_OPTION * n / (mms * 1e-3) / 1e9
        modes[name] = {"ms_per_step": mms, "options_per_s": ws * n / (mms * 1e-3), "gb_per_s": gbs}
    # each mode's results against the FP32 oracle and an FP64 oracle, over the whole batch
    accuracy = {}
    S_h = K_h = T_h = None
    if rank == 0 and not args.no_cpu:
        from nt2_gb300 import synthetic
        S_h, K_h, T_h = synthetic.blackscholes_inputs(n, seed=rank)
        try:
            ref = BSReference(S_h, K_h, T_h)
            for name, prec in (("exact", 0), ("fused", 1), ("fast", 2)):
                make_step(prec)()
                torch.cuda.synchronize()
                accuracy[name] = ref.errors(call.cpu().numpy(), put.cpu().numpy())
            del ref
        except Exception as e:
            accuracy = {"error": repr(e)[:300]}
    from nt2_gb300 import replicas
    value = replicas.job_throughput(n, ws, ms * 1e-3)
    peak, peak_kind = peaks()
    achieved = BYTES_PER_OPTION * n / (ms * 1e-3) / 1e9
    traffic = profiled_traffic("k_blackscholes_f32_n16777216")

    # e2e: host (pinned) buffers through the C ABI, copies inside the timed region
    api.autotune("bs_f32_mapped", n)
    Sh, Kh, Th = (a.cpu().pin_memory() for a in (S, K, T))
    ch = torch.empty(n, dtype=torch.float32).pin_memory()
    ph = torch.empty(n, dtype=torch.float32).pin_memory()
    hs = [a.data_ptr() for a in (Sh, Kh, Th, ch, ph)]

    def e2e_step():
        st = L.nt2cuda_blackscholes_f32_host(hs[0], hs[1], hs[2], R, SIGMA, hs[3], hs[4], n, 0, 0)
        if st:
            raise RuntimeError(f"blackscholes_host status {st}")

    for _ in range(3):
        e2e_step()
    e2e_steps = max(3, min(args.steps, 200))
    # the staged copy pipeline, for comparison (pageable host tables take it automatically)
    Sp, Kp, Tp, cpg, ppg = (torch.empty(n, dtype=torch.float32) for _ in range(5))
    Sp.copy_(Sh); Kp.copy_(Kh); Tp.copy_(Th)
    hsp = [a.data_ptr() for a in (Sp, Kp, Tp, cpg, ppg)]
    st = L.nt2cuda_blackscholes_f32_host(hsp[0], hsp[1], hsp[2], R, SIGMA, hsp[3], hsp[4], n, 0, 0)
    tp0 = time.perf_counter()
    for _ in range(min(e2e_steps, 20)):
        st |= L.nt2cuda_blackscholes_f32_host(hsp[0], hsp[1], hsp[2], R, SIGMA, hsp[3], hsp[4], n, 0, 0)
    staged_pageable_ms = (time.perf_counter() - tp0) * 1e3 / min(e2e_steps, 20)
    if st:
        raise RuntimeError(f"blackscholes_host (pageable) status {st}")
    del Sp, Kp, Tp, cpg, ppg
    barrier(ws)
    te0 = time.perf_counter()
    for _ in range(e2e_steps):
        e2e_step()
    te1 = time.perf_counter()
    e2e_ms = max_over_ranks((te1 - te0) * 1e3 / e2e_steps, ws)
    # results of the e2e path equal the device path's (recomputed: the mode timings reuse call/put)
    step()
    torch.cuda.synchronize()
    same = bool(torch.equal(ch, call.cpu()) and torch.equal(ph, put.cpu()))
    sampler.stop()
    clocks = sampler.summary(t0, t1)

    line = {
        "metric": METRIC, "value": value, "unit": "options/s", "n_gpus": ws, "steps": args.steps,
        "warmup": max(args.warmup, 3), "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": DATA,
        "config": headline_config(n, ws),
        "hbm_frac_measured": achieved / peak, "hbm_frac_nominal": achieved / NOMINAL_HBM_GBS,
        "gb_per_s": achieved,
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "traffic": traffic, "peak_kind": peak_kind,
                     "algorithmic_bytes_per_launch": BYTES_PER_OPTION * n},
        "e2e": {"value": ws * n / (e2e_ms * 1e-3), "unit": "options/s", "h2d_bytes_per_step": 12 * n,
                "d2h_bytes_per_step": 8 * n, "ms_per_step": e2e_ms, "steps": e2e_steps,
                "results_equal_device_path": same,
                "path": "pinned host tables read and written in place by the kernel over NVLink-C2C",
                "pageable_host_tables_ms_per_step": staged_pageable_ms},
        "gpu_launches": args.steps,
        "clocks": clocks,
        "precision_modes": modes,
        "accuracy": accuracy,
        "autotune": tuned,
    }
    peak_v = peak
    for m in modes.values():
        m["hbm_frac_measured"] = m["gb_per_s"] / peak_v
        m["hbm_frac_nominal"] = m["gb_per_s"] / NOMINAL_HBM_GBS
    if rank == 0 and ws == 1 and not args.no_cpu:
        line["cpu_baseline"] = cpu_baseline(S_h, K_h, T_h)
    del S_h, K_h, T_h
    if rank == 0 and ws == 1 and not args.no_serving:
        try:
            line["serving"] = serving_bench()
        except Exception as e:          # the headline number stands without it
            line["serving"] = {"error": repr(e)}
    del S, K, T, call, put, Sh, Kh, Th, ch, ph
    torch.cuda.empty_cache()
    if rank == 0 and ws == 1 and not args.no_configs:
        line["configs"] = config_lines(ws, args.steps, max(args.warmup, 3))
    if rank == 0:
        print(json.dumps(line), flush=True)
    if args.suite and rank == 0:
        for extra in suite(ws):
            print(json.dumps(extra), flush=True)
    if ws > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


CASES = ("bs_exact", "bs_fused", "bs_fast", "bs_fastnormcdf", "bs_demo", "bs_f64", "saxpy", "sdot", "sdot_plain",
         "rgb2grey_u8", "rgb2yuv", "mandelbrot", "trig", "reductions", "scans",
         "inner", "outer", "sigmadelta")


def run_case(name: str, steps: int, warmup: int, autotune: bool = True, part: str | None = None):
    """One configuration alone, for profiling: prints one JSON line (one per part of the
    reductions and scans cases; `part` keeps only the parts whose label contains it)."""
    import torch
    torch.cuda.set_device(0)
    import nt2_gb300.api as api
    api.init(0)
    for line in suite(1, only=name, steps=steps, warmup=warmup, autotune=autotune, part=part):
        print(json.dumps(line), flush=True)


def suite(ws: int, only: str | None = None, steps: int | None = None, warmup: int = 3, autotune: bool = True,
          part: str | None = None):
    """One line per configuration (device time, inputs resident, > L2 or flushed)."""
    import torch
    import nt2_gb300.api as api
    from nt2_gb300 import video
    peak, _ = peaks()
    out = []

    def line(name, ms, bytes_, units, unit):
        gbs = bytes_ / (ms * 1e-3) / 1e9
        return {"config": name, "ms": ms, "gb_per_s": gbs, "hbm_frac_measured": gbs / peak,
                "hbm_frac_nominal": gbs / NOMINAL_HBM_GBS, "value": units / (ms * 1e-3), "unit": unit}

    def want(name):
        return only is None or only == name


    def K(default):
        return steps if steps is not None else default

    if want("saxpy"):
        # four (x, y) pairs (536 MB) visited in turn: every step reads from DRAM, no flush traffic
        n = 1 << 24
        xs = [torch.empty(n, device="cuda") for _ in range(4)]
        ys = [torch.empty(n, device="cuda") for _ in range(4)]
        for i in range(4):
            api.fill_uniform(xs[i], -1, 1, 1 + i)
            api.fill_uniform(ys[i], -1, 1, 11 + i)
        if autotune:
            api.autotune("saxpy_f32", n)
        it = [0]

        def saxpy_step():
            i = it[0] & 3
            it[0] += 1
            api.saxpy(2.5, xs[i], ys[i])
        ms, _, _ = time_device(saxpy_step, K(200), warmup, ws)
        out.append(line("saxpy f32 2^24 (4 rotating copies, 536 MB > L2)", ms, 12 * n, n, "elements/s"))
        del xs, ys
    if want("sdot") or want("sdot_plain"):
        n = 1 << 26
        x = torch.empty(n, device="cuda")
        y = torch.empty(n, device="cuda")
        api.fill_normal(x, 1)
        api.fill_normal(y, 2)
        o = torch.empty(1, device="cuda")
        if want("sdot"):
            ms, _, _ = time_device(lambda: api.dot(x, y, out=o), K(100), warmup, ws)
            out.append(line("sdot f32 2^26 compensated", ms, 8 * n, n, "elements/s"))
        if want("sdot_plain"):
            ms, _, _ = time_device(lambda: api.dot(x, y, compensated=False, out=o), K(100), warmup, ws)
            out.append(line("sdot f32 2^26 plain", ms, 8 * n, n, "elements/s"))
        del x, y
    if want("rgb2grey_u8"):
        # two sets of uint8 planes (2 x 268 MB > L2) visited in turn
        n = 1 << 26
        gen = torch.Generator(device="cuda")
        gen.manual_seed(5)
        sets = [[torch.randint(0, 256, (n,), dtype=torch.uint8, device="cuda", generator=gen) for _ in range(4)]
                for _ in range(2)]
        if autotune:
            api.autotune("rgb2grey_u8", n)
        it = [0]

        def grey_step():
            r, g, b, o = sets[it[0] & 1]
            it[0] += 1
            api.rgb2grey(r, g, b, out=o)
        ms, _, _ = time_device(grey_step, K(200), warmup, ws)
        out.append(line("rgb2grey u8 2^26 pixels (2 rotating sets, 536 MB > L2)", ms, 4 * n, n, "pixels/s"))
        del sets
    if want("rgb2yuv"):
        n = 1 << 24
        sets = []
        for k in range(2):
            planes = [torch.empty(n, device="cuda") for _ in range(3)]
            for j, t in enumerate(planes):
                api.fill_uniform(t, 0, 255, 31 + 3 * k + j)
            sets.append(planes)
        it = [0]

        def yuv_step():
            r, g, b = sets[it[0] & 1]
            it[0] += 1
            api.rgb2yuv(r, g, b)
        ms, _, _ = time_device(yuv_step, K(200), warmup, ws)
        out.append(line("rgb2yuv f32 2^24 pixels (2 rotating sets)", ms, 24 * n, n, "pixels/s"))
        del sets
    if want("mandelbrot"):
        h = w = 1600
        C = torch.empty(h * w, dtype=torch.int32, device="cuda")
        ms, _, _ = time_device(lambda: api.mandelbrot_grid(-1.5, 1.5, -1.5, 1.5, h, w, pack=8, out=C), K(50),
                               warmup, ws)
        counts = C.to(torch.int64).sum().item()
        out.append({"config": "mandelbrot 1600x1600 over [-1.5,1.5]^2, pack 8 (FP32 issue-bound)", "ms": ms,
                    "value": h * w / (ms * 1e-3), "unit": "pixels/s",
                    "counted_trips_per_s": counts / (ms * 1e-3), "mean_count": counts / (h * w)})
    if want("trig"):
        # y = op(x) over 2^24 elements of [-60, 60] (NT2's cover range; packs at the cephes level),
        # 2 rotating inputs of 64/128 MB; 8 (float) or 16 (double) bytes per element
        for dt, tname in ((torch.float32, "f32"), (torch.float64, "f64")):
            n = 1 << 24
            xs = [torch.empty(n, dtype=dt, device="cuda") for _ in range(2)]
            for k, t in enumerate(xs):
                api.fill_uniform(t, -60.0, 60.0, 41 + k)
            y = torch.empty(n, dtype=dt, device="cuda")
            for op in ("sin", "cos", "tan"):
                for simd in (False, True):
                    label = f"{op} {tname} 2^24 [-60,60]{' simd128' if simd else ''}"
                    if part and part not in label:
                        continue
                    it = [0]

                    def trig_step(op=op, simd=simd):
                        x = xs[it[0] & 1]
                        it[0] += 1
                        api.map_(op, x, out=y, simd128=simd)
                    ms, _, _ = time_device(trig_step, K(100), warmup, ws)
                    out.append(line(label, ms, 2 * n * xs[0].element_size(), n, "elements/s"))
            # more functors of the trigonometric, exponential and hyperbolic modules, NT2's scalar form
            for op in ("cot", "sind", "csc", "cbrt", "asinh"):
                label = f"{op} {tname} 2^24 [-60,60]"
                if part and part not in label:
                    continue
                it = [0]

                def op_step(op=op):
                    x = xs[it[0] & 1]
                    it[0] += 1
                    api.map_(op, x, out=y)
                ms, _, _ = time_device(op_step, K(100), warmup, ws)
                out.append(line(label, ms, 2 * n * xs[0].element_size(), n, "elements/s"))
            # exp, log, erfc and the two cdfs, NT2's arithmetic
            for op, lo, hi in (("exp", -60.0, 60.0), ("log", 1e-3, 100.0), ("erfc", -6.0, 6.0), ("normcdf", -6.0, 6.0),
                               ("fastnormcdf", -6.0, 6.0)):
                label = f"{op} {tname} 2^24 [{lo:g},{hi:g}]"
                if part and part not in label:
                    continue
                zs = [torch.empty(n, dtype=dt, device="cuda") for _ in range(2)]
                for k, t in enumerate(zs):
                    api.fill_uniform(t, lo, hi, 61 + k)
                it = [0]

                def map_step(op=op, zs=zs):
                    x = zs[it[0] & 1]
                    it[0] += 1
                    api.map_(op, x, out=y)
                ms, _, _ = time_device(map_step, K(100), warmup, ws)
                out.append(line(label, ms, 2 * n * xs[0].element_size(), n, "elements/s"))
                del zs
            # z = pow(a0, a1) over NT2's cover range: a0 in [0, 100], a1 in [-10, 10];
            # 12 (float) or 24 (double) bytes per element
            label = f"pow {tname} 2^24 a0 in [0,100], a1 in [-10,10]"
            if not part or part in label:
                a1s = [torch.empty(n, dtype=dt, device="cuda") for _ in range(2)]
                for k, t in enumerate(xs):
                    api.fill_uniform(t, 0.0, 100.0, 51 + k)
                for k, t in enumerate(a1s):
                    api.fill_uniform(t, -10.0, 10.0, 61 + k)
                it = [0]

                def pow_step():
                    k = it[0] & 1
                    it[0] += 1
                    api.pow(xs[k], a1s[k], out=y)
                ms, _, _ = time_device(pow_step, K(100), warmup, ws)
                out.append(line(label, ms, 3 * n * xs[0].element_size(), n, "elements/s"))
                del a1s
            del xs, y
    if not (want("inner") or want("outer") or want("reductions") or want("scans") or want("bs_f64") or want("bs_fused") or want("bs_fast")
            or want("bs_exact") or want("bs_fastnormcdf") or want("bs_demo") or want("sigmadelta")):
        return out
    rows, cols = 8192, 4096
    if want("scans"):
        n = 1 << 26
        x = torch.empty(n, device="cuda")
        api.fill_normal(x, 21)
        y = torch.empty(n, device="cuda")
        if part is None or part in "cumsum(x) 2^26":
            ms, _, _ = time_device(lambda: api.cumulative("cumsum", x, n, 1, 1, out=y), K(50), warmup, ws)
            out.append(line("cumsum(x) f32 2^26 vector, compensated (64 KB tiles: aggregate, look-back, rescan from L2)",
                            ms, 8 * n, n, "elements/s"))
        del x, y
        Ts = [torch.empty(rows * cols, device="cuda") for _ in range(2)]
        for i in range(2):
            api.fill_normal(Ts[i], 23 + i)
        o = torch.empty(rows * cols, device="cuda")
        it = [0]
        for dim, note in ((1, "one 32 KB tile per column, single pass"), (2, "one block per 32-row strip walking the columns, TMA-staged single pass")):
            if part is not None and part not in f"cumsum(A,{dim})":
                continue

            def scan_step(dim=dim):
                i = it[0] & 1
                it[0] += 1
                api.cumulative("cumsum", Ts[i], rows, cols, dim, out=o)
            ms, _, _ = time_device(scan_step, K(50), warmup, ws)
            out.append(line(f"cumsum(A,{dim}) 8192x4096 f32 ({note}; 8 B/element algorithmic)", ms,
                            8 * rows * cols, rows * cols, "elements/s"))
        del Ts, o
    if want("reductions"):
        # every reduction of the 8192 x 4096 table along each dimension, four rotating tables
        As = [torch.empty(rows * cols, device="cuda") for _ in range(4)]
        for i in range(4):
            api.fill_normal(As[i], 3 + i)
        it = [0]
        for dim in (1, 2):
            m = cols if dim == 1 else rows
            for op in ("sum", "asum1", "norm2", "mean", "var", "max", "prod", "all"):
                if part is not None and part != f"{op}(A,{dim})":
                    continue
                o = torch.empty(m, dtype=torch.uint8 if op == "all" else torch.float32, device="cuda")

                def red_step(op=op, dim=dim, o=o):
                    i = it[0] & 3
                    it[0] += 1
                    api.reduce(op, As[i], rows, cols, dim, out=o)
                ms, _, _ = time_device(red_step, K(50), warmup, ws)
                out.append(line(f"{op}(A,{dim}) 8192x4096 f32 (4 rotating tables)", ms,
                                4 * rows * cols + o.element_size() * m, rows * cols, "elements/s"))
        del As
    if want("inner") or want("outer"):
        # four 134 MB tables visited in turn (536 MB > L2): every step reads from DRAM
        As = [torch.empty(rows * cols, device="cuda") for _ in range(4)]
        for i in range(4):
            api.fill_normal(As[i], 3 + i)
        oc = torch.empty(cols, device="cuda")
        orow = torch.empty(rows, device="cuda")
        it = [0]

        def fold_step(dim, o):
            def f():
                i = it[0] & 3
                it[0] += 1
                api.sum_colmajor(As[i], rows, cols, dim, out=o)
            return f
        if want("inner"):
            ms, _, _ = time_device(fold_step(1, oc), K(100), warmup, ws)
            out.append(line("inner_fold column sums 8192x4096 f32 compensated (4 rotating tables)", ms,
                            4 * rows * cols + 4 * cols, rows * cols, "elements/s"))
        if want("outer"):
            ms, _, _ = time_device(fold_step(2, orow), K(100), warmup, ws)
            out.append(line("outer_fold row sums 8192x4096 f32 compensated (4 rotating tables)", ms,
                            4 * rows * cols + 4 * rows, rows * cols, "elements/s"))
        del As
    if want("bs_f64"):
        n = 1 << 24
        S = torch.empty(n, dtype=torch.float64, device="cuda")
        Kt = torch.empty(n, dtype=torch.float64, device="cuda")
        T = torch.empty(n, dtype=torch.float64, device="cuda")
        api.fill_uniform(S, 5, 30, 1)
        api.fill_uniform(Kt, 1, 100, 2)
        api.fill_uniform(T, 0.25, 10, 3)
        c = torch.empty_like(S)
        p = torch.empty_like(S)
        ms, _, _ = time_device(lambda: api.blackscholes(S, Kt, T, R, SIGMA, call=c, put=p), K(20), warmup, ws)
        out.append(line("Black-Scholes f64 2^24 (FP64-issue bound)", ms, 40 * n, n, "options/s"))
        del S, Kt, T, c, p
    bs_cases = [("bs_exact", "exact", "normcdf"), ("bs_fused", "fused", "normcdf"), ("bs_fast", "fast", "normcdf"),
                ("bs_fastnormcdf", "exact", "fastnormcdf")]
    if any(want(cn) for cn, _, _ in bs_cases):
        S, Kt, T = bs_tables(1 << 24, 5)
        c = torch.empty_like(S)
        p = torch.empty_like(S)
        for key in ("bs_f32", "bs_f32_fused", "bs_f32_fast"):
            if autotune:
                api.autotune(key, 1 << 24)
        for cn, prec, cdf in bs_cases:
            if not want(cn) or (only is None and cn == "bs_exact"):
                continue
            ms, _, _ = time_device(lambda: api.blackscholes(S, Kt, T, R, SIGMA, call=c, put=p, precision=prec,
                                                            cdf=cdf), K(200), warmup, ws)
            out.append(line(f"Black-Scholes f32 2^24 {prec} {cdf}", ms, 20 * (1 << 24), 1 << 24, "options/s"))
        del S, Kt, T, c, p
    if want("bs_demo"):
        n = 1 << 24
        tabs = [torch.empty(n, device="cuda") for _ in range(5)]
        for t, (lo, hi), sd in zip(tabs, ((5.0, 30.0), (1.0, 100.0), (0.25, 10.0), (0.01, 0.05), (0.1, 0.5)),
                                   (21, 22, 23, 24, 25)):
            api.fill_uniform(t, lo, hi, sd)
        res = torch.empty(n, device="cuda")
        ms, _, _ = time_device(lambda: api.blackscholes_demo(*tabs, out=res), K(50), warmup, ws)
        out.append(line("Black-Scholes demo statement f32 2^24 (5 tables in, 1 out)", ms, 24 * n, n, "options/s"))
        del tabs, res
    if want("sigmadelta"):
        batch = video.make_batch(256, 8, seed=11)
        torch.cuda.synchronize()
        plan = api.SigmaDeltaPlan(batch, 8, init=True)
        ms, _, _ = time_device(plan.launch, K(20), warmup, ws)
        pf = video.pixel_frames(batch, 8, True)
        out.append(line("sigmadelta 256 streams x 8 frames uint8 (graph)", ms, video.bytes_moved(batch, 8, True),
                        pf, "pixel-frames/s"))
        plan.close()
    return out


# ---------------------------------------------------------- reference arm
def run_reference(args):
    """NT2's Black-Scholes statement on the host cores: the oracle's restatement of NT2's
    SIMD+OpenMP path (NT2 itself needs Boost, absent on both machines) over the same 2^24-option
    batch the GPU arm prices, so NT2's spawner takes its OpenMP branch (n > 8 * grain)."""
    ws, rank, _ = dist_env()
    if rank != 0:
        return
    import numpy as np
    from nt2_gb300 import synthetic
    oracle_lib = _oracle()
    L = oracle_lib.load()
    n = N_OPTIONS
    S, K, T = synthetic.blackscholes_inputs(n, seed=0)
    call = np.empty_like(S)
    put = np.empty_like(S)
    th = nt2_threading(L, n, 4)
    steps = args.steps
    for _ in range(max(args.warmup, 3)):
        L.nt2o_bs_f(S, K, T, R, SIGMA, call, put, n, 0, 0)
    t0 = time.perf_counter()
    for _ in range(steps):
        L.nt2o_bs_f(S, K, T, R, SIGMA, call, put, n, 0, 0)
    t1 = time.perf_counter()
    ms = (t1 - t0) * 1e3 / steps
    value = n / (ms * 1e-3)
    desc = (f"the full {n}-option batch each step; NT2's SIMD+OpenMP Black-Scholes path restated in C "
            "(oracle/nt2_oracle.c) because NT2 itself needs Boost, which is absent; scalar+OpenMP, as NT2 "
            f"runs on aarch64 (no Boost.SIMD NEON backend); NT2's spawner rule: grain {th['grain']} elements "
            f"(L2 {th['l2_bytes']} B), parallel={th['parallel']}, {th['threads']} threads")
    print(json.dumps({
        "impl": "reference", "metric": METRIC, "value": value, "unit": "options/s", "n_gpus": ws, "steps": steps,
        "warmup": max(args.warmup, 3), "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": DATA,
        "config": headline_config(n, 1),
        "cpu_baseline": {"value": value, "unit": "options/s", "cores": th["threads"], "kind": "port",
                         "sample": desc, "nt2_threading": th},
        "e2e": {"value": value, "unit": "options/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=2000)
    ap.add_argument("--warmup", type=int, default=20)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--suite", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-serving", action="store_true")
    ap.add_argument("--no-configs", action="store_true", help="skip the other configurations' measurements")
    ap.add_argument("--case", choices=CASES, help="run one configuration alone (for profiling)")
    ap.add_argument("--no-autotune", action="store_true", help="with --case: default launch shapes")
    ap.add_argument("--tuning", default=None, help="tuning-table text to import first (\"key@bucket unroll waves\" lines)")
    ap.add_argument("--part", default=None, help="with --case reductions/scans: one part, e.g. 'var(A,1)'")
    args = ap.parse_args()
    if args.tuning:
        import nt2_gb300.api as api
        api.tuning_import(args.tuning.replace(";", "\n"))
    if args.case:
        run_case(args.case, args.steps, max(args.warmup, 3), autotune=not args.no_autotune, part=args.part)
    elif args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
