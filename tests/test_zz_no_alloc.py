"""nt2cuda_dot_f32_noalloc: the sdot fold for callers that cannot allocate
device memory (their memory belongs to another allocator, or cudaMalloc's
device-wide synchronisation is not acceptable where they run).  Its scratch
is a fixed array in device memory, so it must agree with the allocating
entry point within the sdot tolerance, call after call, reproduce its own
result bit for bit, allocate nothing on a stream it has never seen, and
refuse sizes beyond its fixed limit.

This file is collected last, so a failure here comes after every other test
has run; it also passes on its own in a fresh process."""
import ctypes as C

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

EPS = 2.0 ** -24
MAX_N = 1 << 30


def dot_entry(L, name, x, y, n, comp):
    out = torch.empty(1, dtype=torch.float32, device="cuda")
    st = getattr(L, name)(x.data_ptr(), y.data_ptr(), n, out.data_ptr(), comp,
                          torch.cuda.current_stream().cuda_stream)
    assert st == 0, (name, st, L.nt2cuda_status_string(st))
    torch.cuda.synchronize()
    return float(out.cpu()[0])


@pytest.mark.parametrize("comp", [1, 0])
def test_noalloc_matches_allocating_entry_twice(gpu, oracle, comp):
    import nt2_gb300
    L = nt2_gb300.lib()
    for call, n in enumerate([(1 << 22) + 5, (1 << 24)]):        # two calls in a row, multi-segment folds
        x = torch.empty(n, dtype=torch.float32, device="cuda")
        y = torch.empty(n, dtype=torch.float32, device="cuda")
        gpu.fill_normal(x, 10 + call)
        gpu.fill_normal(y, 20 + call)
        a = dot_entry(L, "nt2cuda_dot_f32_noalloc", x, y, n, comp)
        b = dot_entry(L, "nt2cuda_dot_f32", x, y, n, comp)
        ref, ab = oracle.dot_fp64(x.cpu().numpy(), y.cpu().numpy())
        # the tolerance of the sdot tests: compensated or tree bound plus the product rounding
        tol = (4 * EPS * abs(ref) + 64 * EPS * EPS * n * ab) if comp else (np.log2(n) + 256) * EPS * ab
        assert abs(a - b) <= tol + EPS * ab, (call, a, b)
        assert abs(a - ref) <= tol + EPS * ab, (call, a, ref)


def _scratch_allocations(L):
    c = C.c_ulonglong()
    assert L.nt2cuda_scratch_allocations(C.byref(c)) == 0
    return c.value


def test_noalloc_allocates_nothing_on_a_fresh_stream(gpu):
    """On a stream the library has never seen, nt2cuda_dot_f32 must allocate that
    stream's scratch (the control) while the no-allocation entry point must not;
    its repeated calls also give the same bits."""
    import nt2_gb300
    L = nt2_gb300.lib()
    n = (1 << 22) + 12
    x = torch.empty(n, dtype=torch.float32, device="cuda")
    y = torch.empty(n, dtype=torch.float32, device="cuda")
    gpu.fill_normal(x, 31)
    gpu.fill_normal(y, 32)
    outs = []
    for _ in range(2):
        s = torch.cuda.Stream()
        before = _scratch_allocations(L)
        out = torch.empty(1, dtype=torch.float32, device="cuda")
        assert L.nt2cuda_dot_f32_noalloc(x.data_ptr(), y.data_ptr(), n, out.data_ptr(), 1, s.cuda_stream) == 0
        s.synchronize()
        assert _scratch_allocations(L) == before
        outs.append(out.cpu().numpy().view(np.uint32)[0])
    assert outs[0] == outs[1]
    s = torch.cuda.Stream()
    before = _scratch_allocations(L)
    out = torch.empty(1, dtype=torch.float32, device="cuda")
    assert L.nt2cuda_dot_f32(x.data_ptr(), y.data_ptr(), n, out.data_ptr(), 1, s.cuda_stream) == 0
    s.synchronize()
    assert _scratch_allocations(L) > before


def test_noalloc_small_and_empty(gpu):
    import nt2_gb300
    L = nt2_gb300.lib()
    x = torch.arange(1, 10, dtype=torch.float32, device="cuda")
    y = torch.ones(9, dtype=torch.float32, device="cuda")
    assert dot_entry(L, "nt2cuda_dot_f32_noalloc", x, y, 9, 1) == 45.0
    assert dot_entry(L, "nt2cuda_dot_f32_noalloc", x, y, 0, 1) == 0.0


def test_noalloc_rejects_sizes_beyond_its_scratch(gpu):
    import nt2_gb300
    L = nt2_gb300.lib()
    x = torch.ones(4, dtype=torch.float32, device="cuda")
    out = torch.empty(1, dtype=torch.float32, device="cuda")
    st = L.nt2cuda_dot_f32_noalloc(x.data_ptr(), x.data_ptr(), MAX_N + 1, out.data_ptr(), 1, None)
    assert st == 1                                                   # NT2CUDA_ERR_ARG, nothing launched
