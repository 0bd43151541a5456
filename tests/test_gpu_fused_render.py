"""The fused render pass (uds_render_fused_forward / _backward) against the
separate EWA, compositing and interpolation entry points it replaces:
forward outputs bit-identical, backward gradients equal up to the order of
atomic additions (1e-5 relative L2), and the Splatting module with and
without fusion."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu
DEV = "cuda:0"


def rel_l2(a, b):
    a, b = a.double(), b.double()
    return float((a - b).norm() / b.norm().clamp_min(1e-30))


@pytest.fixture(scope="module")
def mods():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from unbiased_differentiable_splatting_gb300 import library  # noqa: F401
    from unbiased_differentiable_splatting_gb300.cudaExtensions import filtering, interpolation, splatting
    return splatting, filtering, interpolation


def _inputs(seed, B, N, W, H, K, C, aB, sd_scale=1.0):
    rng = np.random.default_rng(seed)
    f = 0.9 * W
    z = rng.uniform(-2.4, -1.6, (B, N))
    pts = np.stack([rng.uniform(-0.5, 0.5, (B, N)) * (-z) * W / f, rng.uniform(-0.5, 0.5, (B, N)) * (-z) * H / f,
                    z], -1)
    n = rng.normal(size=(B, N, 3))
    n[..., 2] = np.abs(n[..., 2]) + 0.8
    n /= np.linalg.norm(n, axis=-1, keepdims=True)
    sd = rng.uniform(0.01, 0.03, size=(1, N, 2)) * sd_scale
    idx = rng.integers(-1, N, size=(B, W, H, K))
    attr = rng.uniform(0.1, 1.0, size=(aB, N, C))
    t = lambda a, d=torch.float32: torch.as_tensor(a, dtype=d, device=DEV).contiguous()  # noqa: E731
    return t(idx, torch.int32), t(pts), t(n), t(sd), t(attr), f


@pytest.mark.parametrize("K,C,aB,sd_scale", [(8, 3, 1, 1.0), (4, 8, 2, 30.0), (13, 3, 2, 30.0)])
def test_fused_matches_separate_ops(mods, K, C, aB, sd_scale):
    splatting, filtering, interpolation = mods
    B, N, W, H = 2, 1500, 40, 32
    idx, pts, nrm, sd, attr, f = _inputs(K + C, B, N, W, H, K, C, aB, sd_scale)
    img, dw, w = splatting.renderForward(W, H, f, idx, pts, nrm, sd, 0.0, attr)
    w_ref = splatting.forward(W, H, f, idx, pts, nrm, sd, 0.0)
    dw_ref = filtering.forward(idx, w_ref, W, H, f, pts, nrm)
    img_ref = interpolation.forward(idx, dw_ref, attr)
    assert torch.equal(w, w_ref) and torch.equal(dw, dw_ref) and torch.equal(img, img_ref)
    if sd_scale > 1:
        assert ((w > 0) & (w < 1)).float().mean() > 0.2  # unclamped weights: EWA gradients flow
    g = torch.randn_like(img)
    gdd = torch.randn_like(dw)
    gww = torch.randn_like(w)
    for gd, gw in ((None, None), (gdd, gww)):
        gp, gn, gs, ga = splatting.renderBackward(W, H, f, g, gd, gw, idx, w, pts, nrm, sd, 0.0, attr)
        gw_ref, ga_ref = interpolation.backward(g, idx, dw_ref, attr)
        if gd is not None:
            gw_ref = gw_ref + gd
        gdw_ref = filtering.backward(idx, w_ref, gw_ref, W, H, f, pts, nrm)
        if gw is not None:
            gdw_ref = gdw_ref + gw
        gp_ref, gn_ref, gs_ref = splatting.backward(W, H, f, gdw_ref.contiguous(), idx, pts, nrm, sd, 0.0)
        torch.cuda.synchronize()
        assert rel_l2(ga, ga_ref) < 1e-5
        for got, ref in ((gp, gp_ref), (gn, gn_ref), (gs, gs_ref)):
            if ref.abs().sum() == 0:
                assert got.abs().sum() == 0
            else:
                assert rel_l2(got, ref) < 1e-5


def test_fused_bad_args(mods):
    splatting = mods[0]
    idx, pts, nrm, sd, attr, f = _inputs(1, 1, 50, 8, 8, 4, 3, 1)
    with pytest.raises(ValueError):
        splatting.renderForward(8, 8, f, idx, pts, nrm, sd, 0.0, attr[:, :10])


@pytest.mark.parametrize("mode", ["forward", "None"])
def test_splatting_fused_equals_unfused(mods, mode):
    from unbiased_differentiable_splatting_gb300 import scenes
    from unbiased_differentiable_splatting_gb300.render import RenderOptions, Splatting
    sc = scenes.harmonic_scene(n=6000, sd_range=(0.01, 0.02), width=64, seed=3)
    r = Splatting(RenderOptions(numSamples=8, precision=0.01, shadingMode=mode), None, 64, 64, sc["focal"], 0.1,
                  100.0, 0.0).to(DEV)
    r.sample_kwargs = {"seed": 21}
    out = []
    for fused in (True, False):
        r.fused = fused
        d = {k: v.to(DEV) for k, v in sc.items() if isinstance(v, torch.Tensor)}
        for k in ("points", "stddevs", "colors", "normals", "cam_positions", "cam_orientations"):
            d[k].requires_grad_(True)
        img, idx, dw = r(d["cam_positions"], d["cam_orientations"], d["points"], d["normals"], d["stddevs"],
                         d["colors"], d["ambient"], d["lamp_directions"], d["lamp_intensities"])
        ((img ** 2).sum() + dw.sum()).backward()
        out.append((img.detach(), idx, dw.detach(), {k: d[k].grad for k in ("points", "stddevs", "colors", "normals",
                                                                             "cam_positions", "cam_orientations")}))
    (i1, x1, d1, g1), (i2, x2, d2, g2) = out
    assert torch.equal(x1, x2) and torch.equal(i1, i2) and torch.equal(d1, d2)
    for k in g2:
        if g2[k] is None:
            assert g1[k] is None, k
        elif g2[k].abs().sum() == 0:
            assert g1[k].abs().sum() == 0, k
        else:
            assert rel_l2(g1[k], g2[k]) < 1e-4, k


def test_opcheck_render_splats(mods):
    splatting = mods[0]
    idx, pts, nrm, sd, attr, f = _inputs(5, 1, 300, 20, 16, 4, 3, 1, 30.0)
    rg = lambda t: t.clone().requires_grad_(True)  # noqa: E731
    torch.library.opcheck(torch.ops.uds.render_splats.default, (20, 16, f, idx, rg(pts), rg(nrm), rg(sd), 0.0,
                                                                rg(attr)))
    img, dw, w = splatting.renderForward(20, 16, f, idx, pts, nrm, sd, 0.0, attr)
    torch.library.opcheck(torch.ops.uds.render_splats_backward.default,
                          (20, 16, f, torch.randn_like(img), None, None, idx, w, pts, nrm, sd, 0.0, attr))
