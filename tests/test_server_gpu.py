"""The continuous-batching request server: each result is the same alone and in
the mix (bit-identical to the single-statement entry point and the oracle),
admission respects the device-memory budget, and waits are bounded."""
import threading
import time

import numpy as np
import pytest
import torch

from nt2_gb300.server import Server, copy_out

pytestmark = pytest.mark.gpu


def pool(n, seed=0):
    S = torch.empty(n, dtype=torch.float32, device="cuda")
    K = torch.empty(n, dtype=torch.float32, device="cuda")
    T = torch.empty(n, dtype=torch.float32, device="cuda")
    import nt2_gb300.api as api
    api.fill_uniform(S, 5, 30, seed + 1)
    api.fill_uniform(K, 1, 100, seed + 2)
    api.fill_uniform(T, 0.25, 10, seed + 3)
    torch.cuda.synchronize()
    return S, K, T


def requests(total, sizes_seed, lo=256, hi=1 << 16, count=200):
    rng = np.random.default_rng(sizes_seed)
    sizes = np.exp(rng.uniform(np.log(lo), np.log(hi), count)).astype(int)
    offs = rng.integers(0, total - hi, count)
    return list(zip(offs.tolist(), sizes.tolist()))


@pytest.mark.parametrize("mode", ["resident", "batched", "launch"])
def test_mix_equals_alone(gpu, oracle, mode):
    coalesce = mode != "launch"
    S, K, T = pool(1 << 20)
    reqs = requests(1 << 20, 1)
    with Server(budget_bytes=256 << 20, max_batch_requests=64, max_inflight_batches=3, mode=mode) as srv:
        tickets = [srv.submit_ptr(S.data_ptr() + 4 * o, K.data_ptr() + 4 * o, T.data_ptr() + 4 * o, 0.02, 0.30, n)
                   for o, n in reqs]
        outs = []
        for t, (o, n) in zip(tickets, reqs):
            c, p = srv.wait(t, 30000)
            outs.append((copy_out(c, n), copy_out(p, n)))
            assert srv.latency_ns(t) > 0
            srv.release(t)
        st = srv.stats()
    assert st["completed"] == len(reqs)
    if coalesce:
        assert st["launches"] < len(reqs)
    else:
        assert st["launches"] == len(reqs)
    Sn, Kn, Tn = (a.cpu().numpy() for a in (S, K, T))
    for (o, n), (c, p) in zip(reqs, outs):
        # alone: the plain entry point on the same sub-range
        ca, pa = gpu.blackscholes(S[o:o + n], K[o:o + n], T[o:o + n], 0.02, 0.30)
        assert torch.equal(c, ca) and torch.equal(p, pa)
        rc, rp = oracle.bs(Sn[o:o + n].copy(), Kn[o:o + n].copy(), Tn[o:o + n].copy(), 0.02, 0.30)
        assert oracle.max_ulp(c.cpu().numpy(), rc)[0] == 0.0
        assert oracle.max_ulp(p.cpu().numpy(), rp)[0] == 0.0


def test_budget_admission_and_release(gpu):
    S, K, T = pool(1 << 20, seed=5)
    n = 1 << 16                                          # 512 KiB of outputs per request
    with Server(budget_bytes=2 << 20, max_batch_requests=16, max_inflight_batches=2) as srv:
        ts = [srv.submit(S[:n], K[:n], T[:n], 0.02, 0.30) for _ in range(12)]
        done = 0
        for t in ts:
            srv.wait(t, 30000)
            st = srv.stats()
            assert st["reserved_bytes"] <= 2 << 20
            srv.release(t)
            done += 1
        st = srv.stats()
        assert st["peak_reserved_bytes"] <= 2 << 20
        assert st["admission_waits"] > 0                 # later requests had to wait for memory
        assert st["completed"] == 12


def test_request_over_budget_rejected(gpu):
    import nt2_gb300
    S, K, T = pool(1 << 16)
    with Server(budget_bytes=64 << 10, max_batch_requests=4, max_inflight_batches=1) as srv:
        with pytest.raises(nt2_gb300.NT2CudaError) as ei:
            srv.submit(S, K, T, 0.02, 0.30)
        assert ei.value.status == 3                      # NT2CUDA_ERR_BUDGET


def test_wait_is_bounded(gpu):
    import nt2_gb300
    S, K, T = pool(1 << 16)
    n = 1 << 14
    with Server(budget_bytes=160 << 10, max_batch_requests=4, max_inflight_batches=1) as srv:
        t1 = srv.submit(S[:n], K[:n], T[:n], 0.02, 0.30)   # 128 KiB: admitted
        t2 = srv.submit(S[:n], K[:n], T[:n], 0.02, 0.30)   # waits for t1's memory
        srv.wait(t1, 30000)
        with pytest.raises(nt2_gb300.NT2CudaError) as ei:
            srv.wait(t2, 50)                              # t1 is never released: t2 cannot be admitted
        assert ei.value.status == 5                      # NT2CUDA_ERR_TIMEOUT
        assert srv.poll(t2) is None
        srv.release(t1)
        srv.wait(t2, 30000)
        srv.release(t2)


def test_concurrent_submitters(gpu, oracle):
    S, K, T = pool(1 << 20, seed=9)
    reqs = requests(1 << 20, 7, count=120)
    results = {}
    with Server(budget_bytes=128 << 20, max_batch_requests=32, max_inflight_batches=3) as srv:
        def client(part):
            for o, n in part:
                t = srv.submit_ptr(S.data_ptr() + 4 * o, K.data_ptr() + 4 * o, T.data_ptr() + 4 * o, 0.02, 0.30, n)
                c, p = srv.wait(t, 30000)
                results[(o, n)] = (copy_out(c, n), copy_out(p, n))
                torch.cuda.synchronize()
                srv.release(t)
        ths = [threading.Thread(target=client, args=(reqs[i::4],)) for i in range(4)]
        for th in ths:
            th.start()
        for th in ths:
            th.join()
        srv.drain(30000)
    for (o, n), (c, p) in results.items():
        ca, pa = gpu.blackscholes(S[o:o + n], K[o:o + n], T[o:o + n], 0.02, 0.30)
        assert torch.equal(c, ca) and torch.equal(p, pa)


def test_replay_trace(gpu, cuda_lib):
    """Native trace replay: every request completes, is released, and has a latency."""
    import numpy as np
    from nt2_gb300.server import Server
    n = 1 << 20
    S, K, T = (torch.empty(n, device="cuda") for _ in range(3))
    gpu.fill_uniform(S, 5, 30, 1)
    gpu.fill_uniform(K, 1, 100, 2)
    gpu.fill_uniform(T, 0.25, 10, 3)
    torch.cuda.synchronize()
    rng = np.random.default_rng(3)
    nreq = 500
    sizes = rng.integers(1, 1 << 16, nreq).astype(np.uint64)
    offs = rng.integers(0, n - (1 << 16), nreq).astype(np.uint64)
    arrivals = np.cumsum(rng.exponential(20e3, nreq)).astype(np.uint64)   # ~50k requests/s
    for coalesce in (True, False):
        with Server(budget_bytes=1 << 28, coalesce=coalesce, max_inflight_batches=3 if coalesce else 1) as srv:
            lat, elapsed = srv.replay(S.data_ptr(), K.data_ptr(), T.data_ptr(), 0.02, 0.3, offs, sizes, arrivals)
            st = srv.stats()
            assert st["completed"] == nreq and st["submitted"] == nreq
            assert st["reserved_bytes"] == 0
            assert np.all(lat > 0) and elapsed > 0
            assert elapsed >= arrivals[-1] * 1e-9


def test_replay_rejects_oversized_request(gpu):
    import numpy as np
    from nt2_gb300.server import Server
    from nt2_gb300._lib import NT2CudaError
    S = torch.empty(1 << 16, device="cuda")
    with Server(budget_bytes=1 << 16) as srv:
        with pytest.raises(NT2CudaError):
            srv.replay(S.data_ptr(), S.data_ptr(), S.data_ptr(), 0.02, 0.3, np.zeros(2, np.uint64),
                       np.array([16, 1 << 16], np.uint64), np.zeros(2, np.uint64))


def test_resident_kernel_leaves_when_idle_and_comes_back(gpu, oracle):
    """The resident kernel's waits are bounded: with no request for its idle bound (20 ms) it
    leaves; the next request launches it again, and results stay bit-exact."""
    S, K, T = pool(1 << 16, seed=4)
    with Server(budget_bytes=64 << 20, mode="resident") as srv:
        outs = []
        for k in range(3):
            o, n = 1000 * k, 4099 + k
            t = srv.submit_ptr(S.data_ptr() + 4 * o, K.data_ptr() + 4 * o, T.data_ptr() + 4 * o, 0.02, 0.30, n)
            c, p = srv.wait(t, 30000)
            outs.append((o, n, copy_out(c, n), copy_out(p, n)))
            srv.release(t)
            time.sleep(0.08)                     # longer than the kernel's idle bound
        st = srv.stats()
    assert st["completed"] == 3
    assert st["launches"] == 3                   # it left after each request and came back
    for o, n, c, p in outs:
        ca, pa = gpu.blackscholes(S[o:o + n], K[o:o + n], T[o:o + n], 0.02, 0.30)
        assert torch.equal(c, ca) and torch.equal(p, pa)


def test_resident_requests_join_the_running_kernel(gpu):
    """Requests submitted while the kernel runs are taken by the same launch."""
    S, K, T = pool(1 << 22, seed=5)
    reqs = requests(1 << 22, 3, lo=1 << 12, hi=1 << 18, count=400)
    with Server(budget_bytes=1 << 30, mode="resident") as srv:
        tickets = []
        for o, n in reqs:
            tickets.append(srv.submit_ptr(S.data_ptr() + 4 * o, K.data_ptr() + 4 * o, T.data_ptr() + 4 * o,
                                          0.02, 0.30, n))
        for t in tickets:
            srv.wait(t, 30000)
            srv.release(t)
        st = srv.stats()
    assert st["completed"] == len(reqs)
    assert st["launches"] <= 2


def test_resident_ring_wraps(gpu):
    """More requests than the ring holds (4096), submitted as fast as possible: ring slots are
    reused only after their request completes, and every request completes, bit-exact."""
    S, K, T = pool(1 << 20, seed=6)
    rng = np.random.default_rng(8)
    count = 10000
    sizes = rng.integers(1, 3000, count)
    offs = rng.integers(0, (1 << 20) - 3000, count)
    with Server(budget_bytes=1 << 30, mode="resident", wait_timeout_ms=20000) as srv:
        tickets = [srv.submit_ptr(S.data_ptr() + 4 * int(o), K.data_ptr() + 4 * int(o), T.data_ptr() + 4 * int(o),
                                  0.02, 0.30, int(n)) for o, n in zip(offs, sizes)]
        check = []
        for k, (t, o, n) in enumerate(zip(tickets, offs, sizes)):
            c, p = srv.wait(t, 20000)
            if k % 997 == 0:
                check.append((int(o), int(n), copy_out(c, int(n)), copy_out(p, int(n))))
            srv.release(t)
        st = srv.stats()
    assert st["completed"] == count
    for o, n, c, p in check:
        ca, pa = gpu.blackscholes(S[o:o + n], K[o:o + n], T[o:o + n], 0.02, 0.30)
        assert torch.equal(c, ca) and torch.equal(p, pa)
