"""The torch.ops.uds registrations on the CPU: every op of the C ABI's
Python surface is registered with the dispatcher and its fake (meta)
implementation gives the output shapes and dtypes of the CUDA op."""
import torch

from unbiased_differentiable_splatting_gb300 import library


def m(*shape, dtype=torch.float32):
    return torch.empty(shape, device="meta", dtype=dtype)


def test_every_op_registered():
    for name in library.OPS:
        assert hasattr(torch.ops.uds, name), name
        assert isinstance(getattr(torch.ops.uds, name).default, torch._ops.OpOverload)


def test_fake_shapes():
    ops = torch.ops.uds
    B, W, H, K, N = 2, 8, 6, 4, 50
    idx = m(B, W, H, K, dtype=torch.int32)
    pts, nrm, sd = m(B, N, 3), m(B, N, 3), m(1, N, 2)
    s = ops.sample(W, H, 10.0, pts, nrm, sd, K, 0.0, 0.01, 3, None, None)
    assert s.shape == (B, W, H, K) and s.dtype == torch.int32
    w = ops.splat_forward(W, H, 10.0, idx, pts, nrm, sd, 0.0)
    assert w.shape == (B, W, H, K) and w.dtype == torch.float32
    gp, gn, gs = ops.splat_backward(W, H, 10.0, w, idx, pts, nrm, sd, 0.0)
    assert (gp.shape, gn.shape, gs.shape) == (pts.shape, nrm.shape, sd.shape)
    assert ops.filter_forward(idx, w, W, H, 10.0, pts, nrm).shape == w.shape
    assert ops.filter_backward(idx, w, w, W, H, 10.0, pts, nrm).shape == w.shape
    img = ops.interp_forward(idx, w, m(1, N, 5))
    assert img.shape == (B, W, H, 5)
    gw, ga = ops.interp_backward(img, idx, w, m(1, N, 5))
    assert gw.shape == w.shape and ga.shape == (1, N, 5)
    M = m(B, 4, 4)
    assert ops.affine_forward(M, m(1, N, 3)).shape == (B, N, 3)
    assert ops.linear_forward(M, m(B, N, 3)).shape == (B, N, 3)
    gM, gv = ops.affine_backward(m(B, N, 3), M, m(1, N, 3))
    assert gM.shape == (B, 4, 4) and gv.shape == (1, N, 3)
    assert ops.view_matrix_forward(m(B, 3), m(B, 4)).shape == (B, 1, 4, 4)
    gp, gq = ops.view_matrix_backward(m(B, 1, 4, 4), m(B, 4))
    assert gp.shape == (B, 3) and gq.shape == (B, 4)
    px = m(B, W, H, 3)
    assert ops.shade_forward(m(B, 2, 3), m(1, 2, 3), px, px).shape == px.shape
    assert [t.shape for t in ops.shade_backward(px, m(B, 2, 3), m(1, 2, 3), px, px)] == [(B, 2, 3), (1, 2, 3),
                                                                                          px.shape, px.shape]
    assert ops.shade_sh_forward(m(1, 3, 9), px, px).shape == px.shape
    assert ops.lambert_forward(m(1, 1, 3), m(B, 2, 3), m(1, 2, 3), pts, m(1, N, 3)).shape == pts.shape
    assert ops.pixel_scatter(idx, m(B, N, 3)).shape == (B, W, H, K, 3)
    assert ops.pixel_gather(idx, m(B, W, H, K, 3), N, True).shape == (B, N, 3)
    nn = ops.nearest(idx, w, m(1, N, 3), 7)
    assert nn.shape == (1, N, 7) and nn.dtype == torch.int32
    losses, gp, gn = ops.nearest_regularizer(nn, m(1, N, 3), m(1, N, 3), 0.5, False)
    assert losses.shape == (2,) and gp.shape == (1, N, 3)
