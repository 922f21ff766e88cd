"""Batched sigma-delta over uneven uint8 streams: bit-exact against the oracle
restatement of demo/sigmadelta/nt2/sigmadelta_nt2.cpp:37-58 (saturating adds)."""
import numpy as np
import pytest
import torch

from nt2_gb300 import video

pytestmark = pytest.mark.gpu


def check_stream(oracle, e, nframes, init, bkg0=None, var0=None):
    torch.cuda.synchronize()
    npix = e["width"] * e["height"]
    frames = e["frames"].cpu().numpy()
    rb, rv, rl = oracle.sigmadelta(frames, e["frame_stride"], npix, nframes, bkg=bkg0, var=var0, init=init)
    gb = e["bkg"].cpu().numpy()
    gv = e["var"].cpu().numpy()
    assert np.array_equal(gb, rb)
    assert np.array_equal(gv, rv)
    nl = nframes - 1 if init else nframes
    gl = e["labels"].cpu().numpy()
    for k in range(nl):
        assert np.array_equal(gl[k * e["label_stride"]:k * e["label_stride"] + npix], rl[k * npix:(k + 1) * npix]), k


def test_uneven_batch_bit_exact(gpu, oracle):
    sizes = [(320, 240), (322, 242), (17, 3), (1, 1), (64, 64), (1920, 1080), (100, 2), (33, 31)]
    batch = [video.make_stream(w, h, 8, seed=i) for i, (w, h) in enumerate(sizes)]
    gpu.sigmadelta_batch(batch, 8, init=True)
    for e in batch:
        check_stream(oracle, e, 8, True)


def test_continue_from_state(gpu, oracle):
    batch = video.make_batch(6, 5, seed=3, sizes=[(320, 240), (640, 480), (18, 18), (1000, 2), (12, 1), (64, 34)])
    gpu.sigmadelta_batch(batch, 5, init=True)
    torch.cuda.synchronize()
    state = [(e["bkg"].cpu().numpy(), e["var"].cpu().numpy()) for e in batch]
    gpu.sigmadelta_batch(batch, 5, init=False)
    for e, (b0, v0) in zip(batch, state):
        check_stream(oracle, e, 5, False, bkg0=b0, var0=v0)


def test_unaligned_strides_take_scalar_path(gpu, oracle):
    e = video.make_stream(50, 7, 4, seed=9, frame_stride=357)   # 350 px, stride not 16-aligned
    gpu.sigmadelta_batch([e], 4, init=True)
    check_stream(oracle, e, 4, True)


def test_graph_plan_matches_direct_launch(gpu, oracle):
    sizes = video.stream_sizes(12, seed=5, lo=(64, 48), hi=(400, 300))
    a = video.make_batch(12, 8, seed=5, sizes=sizes)
    b = video.make_batch(12, 8, seed=5, sizes=sizes)
    gpu.sigmadelta_batch(a, 8, init=True)
    plan = gpu.SigmaDeltaPlan(b, 8, init=True)
    plan.launch()
    torch.cuda.synchronize()
    for ea, eb in zip(a, b):
        for key in ("bkg", "var", "labels"):
            assert torch.equal(ea[key], eb[key])
    plan.close()
    for e in b:
        check_stream(oracle, e, 8, True)


def test_benchmark_batch_bit_exact(gpu, oracle):
    """The batch the benchmark times: 256 streams of 8 frames, sizes log-uniform between
    320x240 and 1920x1080 (seed 11), through the direct batched launch and through the
    CUDA-graph plan; every stream's bkg, var and label planes equal the oracle's."""
    batch = video.make_batch(256, 8, seed=11)
    gpu.sigmadelta_batch(batch, 8, init=True)
    torch.cuda.synchronize()
    direct = [{k: e[k].cpu() for k in ("bkg", "var", "labels")} for e in batch]
    for e in batch:
        check_stream(oracle, e, 8, True)
    for e in batch:                                  # the plan must recompute everything
        for k in ("bkg", "var", "labels"):
            e[k].fill_(0x5a)
    plan = gpu.SigmaDeltaPlan(batch, 8, init=True)
    plan.launch()
    torch.cuda.synchronize()
    plan.close()
    for e, d in zip(batch, direct):
        for k in ("bkg", "var"):
            assert torch.equal(e[k].cpu(), d[k])
        npix = e["width"] * e["height"]
        gl, dl = e["labels"].cpu(), d["labels"]
        for f in range(7):
            lo = f * e["label_stride"]
            assert torch.equal(gl[lo:lo + npix], dl[lo:lo + npix]), f


def test_bad_arguments_rejected(gpu):
    import nt2_gb300
    e = video.make_stream(8, 8, 2, seed=1)
    with pytest.raises(nt2_gb300.NT2CudaError):
        gpu.sigmadelta_batch([e], 0, init=True)
    with pytest.raises(nt2_gb300.NT2CudaError):
        gpu.sigmadelta_batch([e], 1, init=True)          # init needs a frame to start from
    bad = dict(e)
    bad["frame_stride"] = 10                              # smaller than a frame
    with pytest.raises(nt2_gb300.NT2CudaError):
        gpu.sigmadelta_batch([bad], 2, init=True)
