"""world2Camera's fused view-matrix kernels against the reference's tensor
expression (utils.py:11-49): the matrix bit for bit, the pose gradients
against autograd through the expression."""
import pytest
import torch

pytestmark = pytest.mark.gpu
DEV = "cuda:0"


def world2camera_expression(camPositions, camQuaternion):
    B = camPositions.shape[0]
    x, y, z, w = camQuaternion.split(1, dim=-1)
    x2, y2, z2, w2 = x * x, y * y, z * z, w * w
    xy, zw, xz, yw, yz, xw = x * y, z * w, x * z, y * w, y * z, x * w
    row0 = torch.cat([x2 - y2 - z2 + w2, 2 * (xy - zw), 2 * (xz + yw)], dim=-1)
    row1 = torch.cat([2 * (xy + zw), -x2 + y2 - z2 + w2, 2 * (yz - xw)], dim=-1)
    row2 = torch.cat([2 * (xz - yw), 2 * (yz + xw), -x2 - y2 + z2 + w2], dim=-1)
    R = torch.stack([row0, row1, row2], dim=-2)
    top = torch.cat([R, camPositions.reshape(B, 3, 1)], dim=-1)
    bottom = torch.zeros((B, 1, 4), dtype=camPositions.dtype, device=camPositions.device)
    bottom[..., 3] = 1.0
    return torch.cat([top, bottom], dim=-2).unsqueeze(1)


@pytest.mark.parametrize("B", [1, 16, 300])
def test_view_matrix_matches_expression(B):
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from unbiased_differentiable_splatting_gb300.extensions import world2Camera
    g = torch.Generator().manual_seed(B)
    pos = torch.randn(B, 3, generator=g).to(DEV)
    q = torch.nn.functional.normalize(torch.randn(B, 4, generator=g), dim=-1).to(DEV)
    pa, qa = pos.clone().requires_grad_(True), q.clone().requires_grad_(True)
    pb, qb = pos.clone().requires_grad_(True), q.clone().requires_grad_(True)
    Ma = world2Camera(pa, qa)
    Mb = world2camera_expression(pb, qb)
    assert Ma.shape == Mb.shape == (B, 1, 4, 4)
    assert torch.equal(Ma, Mb)
    W = torch.randn(Ma.shape, generator=g).to(DEV)
    (Ma * W).sum().backward()
    (Mb * W).sum().backward()
    torch.testing.assert_close(pa.grad, pb.grad, rtol=0, atol=0)
    torch.testing.assert_close(qa.grad, qb.grad, rtol=1e-5, atol=1e-5)
