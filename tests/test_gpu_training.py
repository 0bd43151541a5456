"""Fused training-step tail against torch: image losses and their
gradients, and the per-splat Adam step with the reference loop's projection."""
import pytest
import torch

pytestmark = pytest.mark.gpu
DEV = "cuda:0"


@pytest.fixture(scope="module")
def tr():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from unbiased_differentiable_splatting_gb300 import training
    return training


@pytest.mark.parametrize("cls,ref", [("L1ImageLoss", lambda x, y: (x - y).abs()),
                                     ("L2ImageLoss", lambda x, y: (x - y).square())])
@pytest.mark.parametrize("reduction", ["sum", "mean"])
def test_image_loss(tr, cls, ref, reduction):
    g = torch.Generator(device=DEV).manual_seed(1)
    x = torch.randn(2, 37, 29, 3, device=DEV, generator=g).requires_grad_(True)
    y = torch.randn(2, 37, 29, 3, device=DEV, generator=g)
    loss, _ = getattr(tr, cls)(reduction)(x, y)
    (3.0 * loss).backward()
    xr = x.detach().clone().requires_grad_(True)
    lr_ = getattr(ref(xr, y), reduction)()
    (3.0 * lr_).backward()
    assert torch.allclose(loss, lr_, rtol=1e-5)
    assert torch.allclose(x.grad, xr.grad, rtol=1e-5, atol=1e-7)


def test_adam_splats_matches_torch(tr):
    from unbiased_differentiable_splatting_gb300.extensions import normalize
    g = torch.Generator(device=DEV).manual_seed(2)
    N, C = 1000, 3
    init = [torch.randn(1, N, 3, device=DEV, generator=g), torch.randn(1, N, 3, device=DEV, generator=g),
            torch.rand(1, N, C, device=DEV, generator=g), 0.01 + 0.02 * torch.rand(1, N, 2, device=DEV, generator=g)]
    init[1] = normalize(init[1])
    ours = [t.clone().requires_grad_(True) for t in init]
    refs = [t.clone().requires_grad_(True) for t in init]
    bounds = (0.005, 0.025)
    opt = tr.SplatAdam(*ours, lr=1e-2, stdDevBound=bounds)
    ropt = torch.optim.Adam(refs, lr=1e-2)
    for it in range(5):
        grads = [torch.randn(t.shape, device=DEV, generator=g) for t in init]
        for t, gr in zip(ours, grads):
            t.grad = gr.clone()
        for t, gr in zip(refs, grads):
            t.grad = gr.clone()
        opt.step()
        ropt.step()
        with torch.no_grad():
            refs[1].set_(normalize(refs[1]))
            refs[3].clamp_(*bounds)
    for a, b in zip(ours, refs):
        assert torch.allclose(a, b, rtol=1e-4, atol=1e-6), float((a - b).abs().max())
