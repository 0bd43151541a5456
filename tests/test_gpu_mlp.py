"""Tensor-core (tcgen05) kernels of the proposal network against torch."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu
DEV = "cuda:0"


@pytest.fixture(scope="module")
def L():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from unbiased_differentiable_splatting_gb300 import _lib
    return _lib.load()


@pytest.mark.parametrize("N,K", [(64, 64), (16, 16), (64, 128), (32, 48)])
def test_mma_probe(L, N, K):
    g = torch.Generator().manual_seed(N * 1000 + K)
    A = torch.randn(128, K, generator=g).to(torch.bfloat16)
    B = torch.randn(N, K, generator=g).to(torch.bfloat16)
    ref = A.float() @ B.float().t()
    res = {}
    for swap in (0, 1):
        C = torch.full((128, N), float("nan"), device=DEV)
        err = torch.zeros(1, dtype=torch.int32, device=DEV)
        Ad, Bd = A.to(DEV).contiguous(), B.to(DEV).contiguous()
        assert L.uds_mma_probe(N, K, Ad.data_ptr(), Bd.data_ptr(), C.data_ptr(), swap, err.data_ptr(),
                               torch.cuda.current_stream().cuda_stream) == 0
        torch.cuda.synchronize()
        assert int(err.item()) == 0
        res[swap] = float((C.cpu() - ref).abs().max() / ref.abs().max())
    print("relative max error by descriptor reading", res)
    assert min(res.values()) < 1e-5, res
    assert res[0] < 1e-5, res  # the reading the library uses


def init_params(n_params, seed=0):
    """The flat parameter array with He-initialised weights."""
    g = torch.Generator().manual_seed(seed)
    P = torch.zeros(n_params)
    o = 0
    for (r, c) in ((64, 16), (64, 64), (64, 64), (16, 64)):
        W = torch.randn(r, c, generator=g) * (2.0 / c) ** 0.5
        if r == 16:
            W[2:] = 0
        P[o:o + r * c] = W.reshape(-1)
        o += r * c
        P[o:o + r] = 0.1 * torch.randn(r, generator=g)
        if r == 16:
            P[o + 2:o + 16] = 0
        o += r
    assert o == n_params
    return P


def torch_forward(P, X):
    """Reference: bf16 operands, fp32 accumulation, bf16 activations."""
    bf = lambda t: t.to(torch.bfloat16).float()  # noqa: E731
    o = 0
    h = bf(X)
    for li, (r, c) in enumerate(((64, 16), (64, 64), (64, 64), (16, 64))):
        W = P[o:o + r * c].reshape(r, c); o += r * c
        b = P[o:o + r]; o += r
        z = h @ bf(W).t() + b
        h = bf(torch.relu(z)) if li < 3 else z
    return h[:, :2]


@pytest.mark.parametrize("R", [1, 128, 1000, 70001])
def test_mlp_forward(L, R):
    n = L.uds_mlp_param_count()
    P = init_params(n, seed=R)
    X = torch.randn(R, 16, generator=torch.Generator().manual_seed(1)) * 2
    ref = torch_forward(P, X)
    out = torch.full((R, 2), float("nan"), device=DEV)
    err = torch.zeros(1, dtype=torch.int32, device=DEV)
    Pd, Xd = P.to(DEV), X.to(DEV)
    assert L.uds_mlp_forward(R, Xd.data_ptr(), Pd.data_ptr(), out.data_ptr(), err.data_ptr(),
                             torch.cuda.current_stream().cuda_stream) == 0
    torch.cuda.synchronize()
    assert int(err.item()) == 0
    d = (out.cpu() - ref).abs().max() / ref.abs().max()
    assert d < 1e-2, float(d)  # bf16 activations: rounding may differ in the last bit
