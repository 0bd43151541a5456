"""Fused per-splat Lambert (forward shading mode) against the reference's
tensor expression (shading.py:12-29), forward and every gradient, for the
broadcast shapes the kernel takes."""
import math

import pytest
import torch

pytestmark = pytest.mark.gpu
DEV = "cuda:0"


def lambert_expression(ambientLight, lampDirections, lampIntensities, normals, diffuse):
    bn, l, _ = lampDirections.shape
    lampDirections = lampDirections.view(bn, l, 1, 3)
    normals = normals.unsqueeze(1)
    ambientIrradiance = ambientLight * diffuse
    bn2, l2, _ = lampIntensities.shape
    radiance = lampIntensities.view(bn2, l2, 1, 3)
    cos = torch.clamp(torch.sum(lampDirections.mul(normals), dim=-1, keepdim=True), 0.0, 1.0)
    irradiance = radiance.mul(cos)
    brdf = diffuse.unsqueeze(1) / math.pi
    return ambientIrradiance + torch.mul(irradiance, brdf).sum(dim=1)


@pytest.mark.parametrize("B,N,L,aB,IB,dB", [(1, 5000, 1, 1, 1, 1), (3, 2049, 1, 1, 1, 1), (2, 777, 3, 2, 2, 2),
                                             (4, 1000, 4, 1, 4, 1), (5, 33, 2, 5, 1, 5)])
def test_lambert_matches_expression(B, N, L, aB, IB, dB):
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from unbiased_differentiable_splatting_gb300 import _lib
    from unbiased_differentiable_splatting_gb300.cudaExtensions import shading
    from unbiased_differentiable_splatting_gb300.extensions import LambertShading
    _lib.load()
    g = torch.Generator().manual_seed(B * 100 + L)
    amb = (0.2 * torch.rand(aB, 1, 3, generator=g)).to(DEV)
    dirs = torch.nn.functional.normalize(torch.randn(B, L, 3, generator=g), dim=-1).to(DEV)
    inten = torch.rand(IB, L, 3, generator=g).to(DEV)
    nrm = torch.nn.functional.normalize(torch.randn(B, N, 3, generator=g), dim=-1).to(DEV)
    dif = torch.rand(dB, N, 3, generator=g).to(DEV)
    assert shading.lambert_shapes(amb, dirs, inten, nrm, dif) == (B, N, L, aB, IB, dB)
    ins_a = [t.clone().requires_grad_(True) for t in (amb, dirs, inten, nrm, dif)]
    ins_b = [t.clone().requires_grad_(True) for t in (amb, dirs, inten, nrm, dif)]
    out_a = LambertShading.apply(*ins_a)
    out_b = lambert_expression(*ins_b)
    assert out_a.shape == out_b.shape
    torch.testing.assert_close(out_a, out_b, rtol=1e-6, atol=1e-6)
    w = torch.randn(out_b.shape, generator=g).to(DEV)
    (out_a * w).sum().backward()
    (out_b * w).sum().backward()
    for ta, tb in zip(ins_a, ins_b):
        # light and ambient gradients are sums over N splats
        torch.testing.assert_close(ta.grad, tb.grad, rtol=1e-4, atol=1e-4 * max(1.0, N / 1000))


def test_lambert_module_uses_fused_kernel():
    """The renderer's Lambert takes the fused path for its shapes and keeps the
    tensor expression for others (e.g. per-splat ambient light)."""
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from unbiased_differentiable_splatting_gb300.cudaExtensions import shading
    from unbiased_differentiable_splatting_gb300.render import Lambert
    amb = torch.full((1, 1, 3), 0.1, device=DEV)
    dirs = torch.nn.functional.normalize(torch.randn(2, 1, 3), dim=-1).to(DEV)
    inten = torch.ones(1, 1, 3, device=DEV)
    nrm = torch.nn.functional.normalize(torch.randn(2, 100, 3), dim=-1).to(DEV)
    dif = torch.rand(1, 100, 3).to(DEV)
    assert shading.lambert_shapes(amb, dirs, inten, nrm, dif) is not None
    torch.testing.assert_close(Lambert()(amb, dirs, inten, nrm, dif),
                               lambert_expression(amb, dirs, inten, nrm, dif), rtol=1e-6, atol=1e-6)
    amb_per_splat = torch.full((1, 100, 3), 0.1, device=DEV)
    assert shading.lambert_shapes(amb_per_splat, dirs, inten, nrm, dif) is None
    torch.testing.assert_close(Lambert()(amb_per_splat, dirs, inten, nrm, dif),
                               lambert_expression(amb_per_splat, dirs, inten, nrm, dif))
