"""cm_mlp_forward_static (intermediates in a fixed __device__ array, nothing allocated) against
cm_mlp_forward on the same device inputs, through the C ABI. Collected last on purpose: it must
pass after every other GPU test in the same process as well as alone in a fresh one."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

MAX_ROWS = 11904  # 8 MiB / 704 B per row, rounded down to 64, for the 22-128-128-19 network


def _err(L):
    return L.cm_last_error().decode()


def _ws_rows(L, net):
    import ctypes
    rows = ctypes.c_int64(-1)
    assert L.cm_diag_mlp_workspace_rows(net._h, ctypes.byref(rows)) == 0, _err(L)
    return rows.value


def test_static_forward_matches_forward_twice(gpu):
    import torch
    L = gpu.lib()
    net = gpu.Mlp(22, 128, 19, seed=7)
    rng = np.random.default_rng(3)
    cases = []
    for n in (300, 5000, MAX_ROWS):
        X = torch.tensor(rng.standard_normal((n, 22)).astype(np.float32), device="cuda")
        Y_ref = torch.zeros((n, 19), dtype=torch.float32, device="cuda")
        Ys = [torch.full((n, 19), float("nan"), dtype=torch.float32, device="cuda") for _ in range(2)]
        cases.append((n, X, Y_ref, Ys))
    torch.cuda.synchronize()
    for n, X, Y_ref, _ in cases:  # the allocating entry point first (it may grow its workspace)
        assert L.cm_mlp_forward(net._h, X.data_ptr(), n, Y_ref.data_ptr()) == 0, _err(L)
    torch.cuda.synchronize()
    n0, X0, _, Ys0 = cases[0]
    assert L.cm_mlp_forward_static(net._h, X0.data_ptr(), n0, Ys0[0].data_ptr()) == 0, _err(L)  # first use
    torch.cuda.synchronize()
    ws0 = _ws_rows(L, net)
    # device-wide free memory: a secondary check that assumes nothing else uses this GPU meanwhile
    free0, _ = torch.cuda.mem_get_info()
    for k, (n, X, Y_ref, Ys) in enumerate(cases):
        for j in range(2):  # two calls in a row
            if k == 0 and j == 0:
                continue
            assert L.cm_mlp_forward_static(net._h, X.data_ptr(), n, Ys[j].data_ptr()) == 0, _err(L)
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    # the network's own workspace did not grow (the primary check), nor did device memory in use
    assert _ws_rows(L, net) == ws0, (ws0, _ws_rows(L, net))
    assert free1 == free0, (free0, free1)
    for n, X, Y_ref, Ys in cases:
        ref = Y_ref.cpu().numpy()
        assert np.isfinite(ref).all()
        for Y in Ys:
            np.testing.assert_allclose(Y.cpu().numpy(), ref, rtol=1e-6, atol=1e-6)


def test_static_forward_rejects(gpu):
    import torch
    L = gpu.lib()
    net = gpu.Mlp(22, 128, 19, seed=7)
    n = MAX_ROWS + 1
    X = torch.zeros((n, 22), dtype=torch.float32, device="cuda")
    Y = torch.zeros((n, 19), dtype=torch.float32, device="cuda")
    torch.cuda.synchronize()
    assert L.cm_mlp_forward_static(net._h, X.data_ptr(), n, Y.data_ptr()) == -1
    assert str(MAX_ROWS) in _err(L)
    Xh = np.zeros((8, 22), np.float32)
    Yh = np.zeros((8, 19), np.float32)
    assert L.cm_mlp_forward_static(net._h, Xh.ctypes.data, 8, Yh.ctypes.data) == -1
    assert "device arrays" in _err(L)
    assert L.cm_mlp_forward_static(net._h, X.data_ptr(), 0, Y.data_ptr()) == 0
