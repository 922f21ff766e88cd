"""The host restatement of the seeded uniform generator gives the device's tables bit for bit,
so the CPU baseline and the oracle checks of the benchmark see the GPU's inputs."""
import numpy as np
import pytest
import torch

from nt2_gb300 import synthetic

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("dtype,lo,hi,seed,n", [
    (torch.float32, 5.0, 30.0, 1, (1 << 20) + 3),
    (torch.float32, 1.0, 100.0, 2, 4097),
    (torch.float32, -1.0, 1.0, 77, 1 << 16),
    (torch.float64, 0.25, 10.0, 3, (1 << 18) + 1),
])
def test_host_generator_equals_device(gpu, dtype, lo, hi, seed, n):
    x = torch.empty(n, dtype=dtype, device="cuda")
    gpu.fill_uniform(x, lo, hi, seed)
    dev = x.cpu().numpy()
    host = (synthetic.uniform_f32 if dtype == torch.float32 else synthetic.uniform_f64)(n, lo, hi, seed)
    assert np.array_equal(dev.view(np.uint32 if dtype == torch.float32 else np.uint64),
                          host.view(np.uint32 if dtype == torch.float32 else np.uint64))
