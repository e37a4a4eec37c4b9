"""The tcgen05 tensor-core path (shared-memory operand layout, descriptors, TMEM accumulator and
its read-back) that the learned macro step uses, on one tile against a host product of the same
BF16 operands (FP32 accumulation of at most 128 products: relative error <= 1e-5)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("n,k", [(128, 32), (128, 128), (32, 128), (64, 64)])
def test_umma_tile_matches_host_product(gpu, n, k):
    import torch
    L = gpu.lib()
    g = torch.Generator().manual_seed(n * 1000 + k)
    A = torch.randn(128, k, generator=g).to(torch.bfloat16)
    B = torch.randn(n, k, generator=g).to(torch.bfloat16)
    ref = A.double() @ B.double().T
    dA, dB = A.cuda(), B.cuda()
    D = torch.full((128, n), float("nan"), dtype=torch.float32, device="cuda")
    torch.cuda.synchronize()
    assert L.cm_diag_umma_tile(dA.data_ptr(), dB.data_ptr(), n, k, D.data_ptr(), None) == 0
    got = D.cpu().double()
    err = (got - ref).abs().max().item() / ref.abs().max().item()
    assert err < 1e-5, err
