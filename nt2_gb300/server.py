"""Python handle on the nt2cuda continuous-batching request server."""
from __future__ import annotations

import ctypes as C

import torch

from ._lib import NT2CudaError, ServerConfig, ServerStats, check, lib

NOT_READY = 7
TIMEOUT = 5


class Server:
    """Black-Scholes request server (float32; inputs are device tables)."""

    MODES = {"launch": 0, "batched": 1, "resident": 2}

    def __init__(self, budget_bytes: int = 40 << 30, max_batch_requests: int = 4096,
                 max_inflight_batches: int = 3, coalesce: bool = True, fused: bool = False,
                 cdf: str = "normcdf", wait_timeout_ms: int = 60000, precision: str | None = None,
                 spin_us: int = 0, mode: str | None = None):
        """mode: "resident" (one kernel stays on the device and drains a request ring),
        "batched" (one launch per step over the admitted requests) or "launch" (one launch
        per request); without it, coalesce picks "batched" or "launch"."""
        prec = {"exact": 0, "fused": 1, "fast": 2}[precision] if precision else int(fused)
        co = self.MODES[mode] if mode else int(coalesce)
        cfg = ServerConfig(budget_bytes, max_batch_requests, max_inflight_batches, co, prec,
                           {"normcdf": 0, "fastnormcdf": 1}[cdf], wait_timeout_ms, spin_us)
        self._h = C.c_void_p()
        check(lib().nt2cuda_server_create(C.byref(cfg), C.byref(self._h)), "server_create")

    def submit(self, S: torch.Tensor, K: torch.Tensor, T: torch.Tensor, r: float, sigma: float) -> int:
        t = C.c_uint64()
        check(lib().nt2cuda_server_submit(self._h, S.data_ptr(), K.data_ptr(), T.data_ptr(), r, sigma, S.numel(),
                                          C.byref(t)), "server_submit")
        return t.value

    def submit_ptr(self, S: int, K: int, T: int, r: float, sigma: float, n: int) -> int:
        t = C.c_uint64()
        check(lib().nt2cuda_server_submit(self._h, S, K, T, r, sigma, n, C.byref(t)), "server_submit")
        return t.value

    def wait(self, ticket: int, timeout_ms: int = -1):
        """Device pointers (call, put) of a finished request."""
        c, p = C.c_void_p(), C.c_void_p()
        check(lib().nt2cuda_server_wait(self._h, ticket, timeout_ms, C.byref(c), C.byref(p)), "server_wait")
        return c.value, p.value

    def poll(self, ticket: int):
        c, p = C.c_void_p(), C.c_void_p()
        st = lib().nt2cuda_server_poll(self._h, ticket, C.byref(c), C.byref(p))
        if st == NOT_READY:
            return None
        check(st, "server_poll")
        return c.value, p.value

    def latency_ns(self, ticket: int) -> int:
        v = C.c_uint64()
        check(lib().nt2cuda_server_latency_ns(self._h, ticket, C.byref(v)), "server_latency")
        return v.value

    def release(self, ticket: int) -> None:
        check(lib().nt2cuda_server_release(self._h, ticket), "server_release")

    def drain(self, timeout_ms: int = -1) -> None:
        check(lib().nt2cuda_server_drain(self._h, timeout_ms), "server_drain")

    def replay(self, S: int, K: int, T: int, r: float, sigma: float, offsets, sizes, arrival_ns):
        """Replay a trace natively (nt2cuda_server_replay): request i uses the tables at device
        addresses S/K/T + 4*offsets[i] with sizes[i] options and arrives arrival_ns[i] after the start.
        Returns (per-request latency in ns as a numpy array, elapsed seconds)."""
        import numpy as np
        off = np.ascontiguousarray(offsets, dtype=np.uint64)
        siz = np.ascontiguousarray(sizes, dtype=np.uint64)
        arr = np.ascontiguousarray(arrival_ns, dtype=np.uint64)
        lat = np.zeros(off.size, dtype=np.uint64)
        el = C.c_uint64()
        check(lib().nt2cuda_server_replay(self._h, S, K, T, r, sigma, off.size, off.ctypes.data, siz.ctypes.data,
                                          arr.ctypes.data, lat.ctypes.data, C.byref(el)), "server_replay")
        return lat, el.value * 1e-9

    def stats(self) -> dict:
        s = ServerStats()
        check(lib().nt2cuda_server_get_stats(self._h, C.byref(s)), "server_stats")
        return {k: getattr(s, k) for k, _ in ServerStats._fields_}

    def close(self) -> None:
        if self._h:
            lib().nt2cuda_server_destroy(self._h)
            self._h = C.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def copy_out(ptr: int, n: int, device: torch.device | None = None) -> torch.Tensor:
    """Copy n float32 values from a server output slot into a new CUDA tensor.

    Returns after the copy has completed, so the slot may be released at once."""
    dst = torch.empty(n, dtype=torch.float32, device=device or "cuda")
    stream = torch.cuda.current_stream()
    check(lib().nt2cuda_memcpy_d2d(dst.data_ptr(), ptr, n * 4, stream.cuda_stream), "copy_out")
    stream.synchronize()
    return dst


__all__ = ["Server", "copy_out", "NT2CudaError"]
