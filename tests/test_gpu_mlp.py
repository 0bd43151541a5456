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


def torch_loss(P, X, target):
    """Mean cross-entropy of the torch reference (bf16-rounded operands)."""
    logits = torch_forward(P, X)
    logq = torch.log_softmax(logits, -1)
    return -(target * logq[:, 0] + (1 - target) * logq[:, 1]).mean()


@pytest.mark.parametrize("R", [128, 5000])
def test_mlp_grad(L, R):
    n = L.uds_mlp_param_count()
    P = init_params(n, seed=7)
    g = torch.Generator().manual_seed(R)
    X = torch.randn(R, 16, generator=g)
    target = torch.rand(R, generator=g)
    Pr = P.clone().requires_grad_(True)
    loss = torch_loss(Pr, X, target)
    loss.backward()
    ref = Pr.grad
    G = torch.zeros(n, device=DEV)
    lo = torch.zeros(1, device=DEV)
    err = torch.zeros(1, dtype=torch.int32, device=DEV)
    Pd, Xd, td = P.to(DEV), X.to(DEV), target.to(DEV)
    ws = torch.empty(L.uds_mlp_grad_workspace_size(R), dtype=torch.uint8, device=DEV)
    assert L.uds_mlp_grad(R, Xd.data_ptr(), td.data_ptr(), Pd.data_ptr(), G.data_ptr(), lo.data_ptr(),
                          err.data_ptr(), ws.data_ptr(), ws.numel(), torch.cuda.current_stream().cuda_stream) == 0
    torch.cuda.synchronize()
    assert int(err.item()) == 0
    assert abs(float(lo.item()) - float(loss.detach())) < 1e-3 * abs(float(loss.detach())) + 1e-4
    Gc = G.cpu()
    o = 0
    for (r, c) in ((64, 16), (64, 64), (64, 64), (16, 64)):
        for size in (r * c, r):
            a, b = Gc[o:o + size], ref[o:o + size]
            rel = float((a - b).norm() / (b.norm() + 1e-12))
            assert rel < 0.03, (o, size, rel)  # bf16 rounding of the backward operands
            o += size


def test_mlp_training_reduces_loss(L):
    """A few hundred Adam steps on a smooth target drive the loss down."""
    n = L.uds_mlp_param_count()
    P = init_params(n, seed=3).to(DEV)
    m1 = torch.zeros(n, device=DEV)
    m2 = torch.zeros(n, device=DEV)
    G = torch.zeros(n, device=DEV)
    g = torch.Generator(device=DEV).manual_seed(0)
    X = torch.randn(20000, 16, device=DEV, generator=g)
    target = torch.sigmoid(2.0 * X[:, 0] - X[:, 1] + 0.5 * X[:, 2] * X[:, 3])
    err = torch.zeros(1, dtype=torch.int32, device=DEV)
    s = torch.cuda.current_stream().cuda_stream
    losses = []
    ws = torch.empty(L.uds_mlp_grad_workspace_size(X.shape[0]), dtype=torch.uint8, device=DEV)
    for step in range(1, 301):
        lo = torch.zeros(1, device=DEV)
        assert L.uds_mlp_grad(X.shape[0], X.data_ptr(), target.data_ptr(), P.data_ptr(), G.data_ptr(), lo.data_ptr(),
                              err.data_ptr(), ws.data_ptr(), ws.numel(), s) == 0
        assert L.uds_mlp_adam(P.data_ptr(), G.data_ptr(), m1.data_ptr(), m2.data_ptr(), step, 3e-3, 0.9, 0.999,
                              1e-8, s) == 0
        if step in (1, 300):
            losses.append(float(lo.item()))
    assert int(err.item()) == 0
    # entropy floor of the soft targets
    floor = float(-(target * target.log() + (1 - target) * (1 - target).log()).mean())
    assert losses[1] - floor < 0.25 * (losses[0] - floor), (losses, floor)


def pack_tiles(X):
    """Rows (R,16) -> bf16 operand tiles (128 rows x 16 per 4096 bytes)."""
    R = X.shape[0]
    tiles = (R + 127) // 128
    buf = torch.zeros(tiles * 2048, dtype=torch.bfloat16, device=X.device)
    r = torch.arange(R, device=X.device)[:, None]
    k = torch.arange(16, device=X.device)[None, :]
    rr = r % 128
    idx = (r // 128) * 2048 + (rr // 8) * 128 + (k // 8) * 64 + (rr % 8) * 8 + (k % 8)
    buf[idx.reshape(-1)] = X.to(torch.bfloat16).reshape(-1)
    return buf


@pytest.mark.parametrize("R,Rdev", [(1, 1), (1000, 1000), (70001, 70001), (70001, 12345)])
def test_mlp_forward_tiles_bulk_copy(L, R, Rdev):
    """The bulk-copy (TMA engine) variant on pre-laid-out bf16 tiles gives the
    same logits as the fp32-row variant, for the device-side row count."""
    n = L.uds_mlp_param_count()
    P = init_params(n, seed=R).to(DEV)
    X = (torch.randn(R, 16, generator=torch.Generator().manual_seed(2)) * 2).to(DEV)
    s = torch.cuda.current_stream().cuda_stream
    err = torch.zeros(1, dtype=torch.int32, device=DEV)
    ref = torch.full((R, 2), float("nan"), device=DEV)
    assert L.uds_mlp_forward(R, X.data_ptr(), P.data_ptr(), ref.data_ptr(), err.data_ptr(), s) == 0
    tiles = pack_tiles(X)
    cnt = torch.tensor([Rdev], dtype=torch.int32, device=DEV)
    out = torch.full((R, 2), float("nan"), device=DEV)
    assert L.uds_mlp_forward_tiles(R, cnt.data_ptr(), tiles.data_ptr(), P.data_ptr(), out.data_ptr(),
                                   err.data_ptr(), s) == 0
    torch.cuda.synchronize()
    assert int(err.item()) == 0
    assert torch.equal(out[:Rdev], ref[:Rdev])
    assert torch.isnan(out[Rdev:]).all()
