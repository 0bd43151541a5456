"""torch.ops.uds on the GPU: torch.library.opcheck of every registered op
(schema, fake tensor, autograd registration, AOT dispatch with dynamic
shapes) on small inputs, and torch.compile of the render chain and of the
Splatting module with fullgraph=True (no graph break) matching eager."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu
DEV = "cuda:0"


@pytest.fixture(scope="module")
def ops():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from unbiased_differentiable_splatting_gb300 import library  # noqa: F401
    return torch.ops.uds


def _scene(seed=0, B=1, N=400, W=24, H=20, f=22.0):
    rng = np.random.default_rng(seed)
    z = rng.uniform(-2.4, -1.6, (B, N))
    pts = np.stack([rng.uniform(-0.5, 0.5, (B, N)) * (-z) * W / f, rng.uniform(-0.5, 0.5, (B, N)) * (-z) * H / f,
                    z], -1)
    n = rng.normal(size=(B, N, 3))
    n[..., 2] = np.abs(n[..., 2]) + 0.8
    n /= np.linalg.norm(n, axis=-1, keepdims=True)
    sd = rng.uniform(0.01, 0.03, size=(1, N, 2))
    t = lambda a: torch.as_tensor(a, dtype=torch.float32, device=DEV).contiguous()  # noqa: E731
    return t(pts), t(n), t(sd), W, H, f


def _check(op, args):
    torch.library.opcheck(op, args)


def test_opcheck_sampler_and_render_chain(ops):
    pts, nrm, sd, W, H, f = _scene()
    nb = torch.where(nrm[..., 2:] > 0, -nrm, nrm).contiguous()
    _check(ops.sample.default, (W, H, f, pts, nb, sd, 4, 0.0, 0.01, 7, None, None))
    idx = ops.sample(W, H, f, pts, nb, sd, 4, 0.0, 0.01, 7, None, None)
    assert (idx >= 0).any()
    p, n, s = (x.clone().requires_grad_(True) for x in (pts, nrm, sd))
    _check(ops.splat_forward.default, (W, H, f, idx, p, n, s, 0.0))
    _check(ops.ewa_weights.default, (W, H, f, idx, p, n, s, 0.0))
    w = ops.splat_forward(W, H, f, idx, pts, nrm, sd, 0.0)
    _check(ops.splat_backward.default, (W, H, f, torch.ones_like(w), idx, pts, nrm, sd, 0.0))
    _check(ops.filter_forward.default, (idx, w.clone().requires_grad_(True), W, H, f, pts, nrm))
    dw = ops.filter_forward(idx, w, W, H, f, pts, nrm)
    _check(ops.filter_backward.default, (idx, w, torch.ones_like(w), W, H, f, pts, nrm))
    col = torch.rand((1, pts.shape[1], 3), device=DEV)
    _check(ops.interp_forward.default, (idx, dw.clone().requires_grad_(True), col.clone().requires_grad_(True)))
    img = ops.interp_forward(idx, dw, col)
    _check(ops.interp_backward.default, (torch.ones_like(img), idx, dw, col))


def test_opcheck_transform_and_shading(ops):
    B, N = 2, 300
    M = torch.randn(B, 4, 4, device=DEV)
    v = torch.randn(1, N, 3, device=DEV)
    for name in ("affine", "linear"):
        _check(getattr(ops, f"{name}_forward").default, (M.clone().requires_grad_(True), v.clone().requires_grad_(True)))
        _check(getattr(ops, f"{name}_backward").default, (torch.randn(B, N, 3, device=DEV), M, v))
    pos = torch.randn(B, 3, device=DEV)
    q = torch.nn.functional.normalize(torch.randn(B, 4, device=DEV), dim=-1)
    _check(ops.view_matrix_forward.default, (pos.clone().requires_grad_(True), q.clone().requires_grad_(True)))
    _check(ops.view_matrix_backward.default, (torch.randn(B, 1, 4, 4, device=DEV), q))
    px = torch.nn.functional.normalize(torch.randn(B, 6, 5, 3, device=DEV), dim=-1)
    dif = torch.rand(B, 6, 5, 3, device=DEV)
    dirs = torch.nn.functional.normalize(torch.randn(B, 2, 3, device=DEV), dim=-1)
    inten = torch.rand(1, 2, 3, device=DEV)
    rg = lambda t: t.clone().requires_grad_(True)  # noqa: E731
    _check(ops.shade_forward.default, (rg(dirs), rg(inten), rg(px), rg(dif)))
    _check(ops.shade_backward.default, (torch.randn_like(px), dirs, inten, px, dif))
    coef = torch.randn(1, 3, 9, device=DEV)
    _check(ops.shade_sh_forward.default, (rg(coef), rg(px), rg(dif)))
    _check(ops.shade_sh_backward.default, (torch.randn_like(px), coef, px, dif))
    nrm = torch.nn.functional.normalize(torch.randn(B, N, 3, device=DEV), dim=-1)
    alb = torch.rand(1, N, 3, device=DEV)
    amb = torch.rand(1, 1, 3, device=DEV)
    _check(ops.lambert_forward.default, (rg(amb), rg(dirs), rg(inten), rg(nrm), rg(alb)))
    _check(ops.lambert_backward.default, (torch.randn(B, N, 3, device=DEV), amb, dirs, inten, nrm, alb))


def test_opcheck_per_splat_consumers(ops):
    pts, nrm, sd, W, H, f = _scene(seed=2)
    nb = torch.where(nrm[..., 2:] > 0, -nrm, nrm).contiguous()
    idx = ops.sample(W, H, f, pts, nb, sd, 4, 0.0, 0.01, 3, None, None)
    vals = torch.rand(1, pts.shape[1], 3, device=DEV)
    _check(ops.pixel_scatter.default, (idx, vals.clone().requires_grad_(True)))
    _check(ops.pixel_gather.default, (idx, torch.rand(*idx.shape, 3, device=DEV), pts.shape[1], True))
    w = ops.splat_forward(W, H, f, idx, pts, nrm, sd, 0.0)
    _check(ops.nearest.default, (idx, w, pts, 5))
    nn = ops.nearest(idx, w, pts, 5)
    _check(ops.nearest_regularizer.default, (nn, pts, nrm, 0.5, False))


def test_compile_fullgraph_matches_eager(ops):
    """The render chain and the Splatting module trace into one graph each
    (torch.compile, fullgraph=True, aot_eager backend: the CUDA ops run as
    they are) and give the eager results."""
    from unbiased_differentiable_splatting_gb300 import scenes
    from unbiased_differentiable_splatting_gb300.render import RenderOptions, Splatting
    pts, nrm, sd, W, H, f = _scene(seed=5)
    nb = torch.where(nrm[..., 2:] > 0, -nrm, nrm).contiguous()
    idx = ops.sample(W, H, f, pts, nb, sd, 4, 0.0, 0.01, 9, None, None)
    col = torch.rand((1, pts.shape[1], 3), device=DEV)

    def chain(idx, p, n, s, c):
        w = ops.splat_forward(W, H, f, idx, p, n, s, 0.0)
        dw = ops.filter_forward(idx, w, W, H, f, p, n)
        return ops.interp_forward(idx, dw, c)

    compiled = torch.compile(chain, backend="aot_eager", fullgraph=True)
    p1, p2 = pts.clone().requires_grad_(True), pts.clone().requires_grad_(True)
    a = chain(idx, p1, nrm, sd, col)
    b = compiled(idx, p2, nrm, sd, col)
    assert torch.equal(a, b)
    a.sum().backward()
    b.sum().backward()
    torch.testing.assert_close(p1.grad, p2.grad, rtol=1e-5, atol=1e-6)

    sc = scenes.harmonic_scene(n=3000, sd_range=(0.01, 0.02), width=32, seed=1)
    d = {k: v.to(DEV) for k, v in sc.items() if isinstance(v, torch.Tensor)}
    r = Splatting(RenderOptions(numSamples=4, precision=0.01, shadingMode="forward"), None, 32, 32, sc["focal"], 0.1,
                  100.0, 0.0).to(DEV)
    r.sample_kwargs = {"seed": 11}
    args = (d["cam_positions"], d["cam_orientations"], d["points"], d["normals"], d["stddevs"], d["colors"],
            d["ambient"], d["lamp_directions"], d["lamp_intensities"])
    img_e, idx_e, dw_e = r(*args)
    img_c, idx_c, dw_c = torch.compile(r, backend="aot_eager", fullgraph=True)(*args)
    assert torch.equal(idx_e, idx_c)
    torch.testing.assert_close(img_c, img_e, rtol=1e-6, atol=1e-7)


def test_backface_kernel_matches_where(ops):
    """uds::backface against the reference's torch.where expression, forward
    and backward (world normals shared by the views: gradients summed)."""
    B, N = 3, 1000
    cam = torch.randn(B, N, 3, device=DEV)
    cam[0, :5, 2] = 0.0
    nrm = torch.randn(1, N, 3, device=DEV)
    fc, fw = ops.backface(cam, nrm)
    facing = cam[..., 2:] > 0
    assert torch.equal(fc, torch.where(facing, -cam, cam))
    assert torch.equal(fw, torch.where(facing, -nrm, nrm))
    (fc_only,) = ops.backface(cam, None)
    assert torch.equal(fc_only, fc)
    c1, n1 = cam.clone().requires_grad_(True), nrm.clone().requires_grad_(True)
    c2, n2 = cam.clone().requires_grad_(True), nrm.clone().requires_grad_(True)
    g1, g2 = torch.randn(B, N, 3, device=DEV), torch.randn(B, N, 3, device=DEV)
    a, b = ops.backface(c1, n1)
    ((a * g1).sum() + (b * g2).sum()).backward()
    f2 = c2[..., 2:].detach() > 0
    ((torch.where(f2, -c2, c2) * g1).sum() + (torch.where(f2, -n2, n2) * g2).sum()).backward()
    assert torch.equal(c1.grad, c2.grad)
    torch.testing.assert_close(n1.grad, n2.grad, rtol=1e-6, atol=1e-6)
    _check(ops.backface.default, (cam.clone().requires_grad_(True), nrm.clone().requires_grad_(True)))
    _check(ops.backface_backward.default, (cam, g1, g2, 1))
