"""nearestsamples.nearest on the GPU against the oracle, and the
nearest-sample regulariser on a rendered view."""
import numpy as np
import pytest
import torch

import oracle

pytestmark = pytest.mark.gpu
DEV = "cuda:0"


@pytest.fixture(scope="module")
def ns():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from unbiased_differentiable_splatting_gb300.cudaExtensions import nearestsamples
    return nearestsamples


@pytest.mark.parametrize("M", [1, 7, 32])
def test_nearest_matches_oracle(ns, M):
    rng = np.random.default_rng(M)
    B, W, H, K, N = 2, 40, 30, 8, 900
    idx = rng.integers(-1, N, size=(B, W, H, K)).astype(np.int32)
    idx[rng.random(idx.shape) < 0.1] = 5  # repeated splats within pixels
    w = rng.random((B, W, H, K)).astype(np.float32)
    w[..., 3] = w[..., 2]  # ties in the surface choice
    pts = rng.normal(size=(1, N, 3)).astype(np.float32)
    got = ns.nearest(torch.as_tensor(idx).to(DEV), torch.as_tensor(w).to(DEV), torch.as_tensor(pts).to(DEV), M)
    ref = oracle.nearest_samples(idx, w, pts, M)
    np.testing.assert_array_equal(got.cpu().numpy()[0], ref)
    assert (ref >= 0).any()


def _regularizer_fp64(nearest, pts, nrm, sigma):
    """NearestSamplesRegularizer (regularizier.py:119-175) restated in FP64
    numpy: per-splat normal and plane losses, and their gradients w.r.t. the
    splat's own normal and point (weights and mean normals held constant)."""
    n = nearest[0]
    P = pts[0].astype(np.float64)
    Nn = nrm[0].astype(np.float64)
    mask = (n > 0)[..., None].astype(np.float64)
    j = np.clip(n, 0, None)
    Pj, Nj = P[j], Nn[j]
    gauss = lambda x: np.exp(-x ** 2 / sigma ** 2)  # noqa: E731
    w = mask * gauss(np.linalg.norm(Nn[:, None] - Nj, axis=-1))[..., None] * \
        gauss(np.linalg.norm(P[:, None] - Pj, axis=-1))[..., None]
    inv = 1.0 / (w.sum(1) + 1e-4)
    F = (w * Nj).sum(1)
    filt = F / (np.linalg.norm(F, axis=-1, keepdims=True) + 1e-4)
    pm = np.clip(mask.sum(1), 0, 1)
    D = (w * ((P[:, None] - Pj) * Nj).sum(-1, keepdims=True)).sum(1)
    plane = (inv * D) ** 2
    normal = pm * ((filt - Nn) ** 2).sum(-1, keepdims=True)
    return normal[:, 0], plane[:, 0], 2 * inv ** 2 * D * F, -2 * pm * (filt - Nn)


@pytest.mark.parametrize("reduction", ["sum", "mean"])
def test_regularizer_on_render(ns, reduction):
    """The regulariser's kernel on a rendered view's nearest lists against the
    FP64 restatement: both losses and the points' / normals' gradients."""
    from unbiased_differentiable_splatting_gb300 import scenes
    from unbiased_differentiable_splatting_gb300.regularizers import NearestSamplesRegularizer
    from unbiased_differentiable_splatting_gb300.render import RenderOptions, Splatting
    sc = scenes.harmonic_scene(n=4000, sd_range=(0.01, 0.02), width=64, seed=2)
    d = {k: v.to(DEV) for k, v in sc.items() if isinstance(v, torch.Tensor)}
    r = Splatting(RenderOptions(numSamples=8, precision=0.01), None, 64, 64, sc["focal"], 0.1, 100.0, 0.0).to(DEV)
    pts = d["points"].clone().requires_grad_(True)
    nrm = d["normals"].clone().requires_grad_(True)
    img, idx, dw = r(d["cam_positions"], d["cam_orientations"], pts, nrm, d["stddevs"], d["colors"], d["ambient"],
                     d["lamp_directions"], d["lamp_intensities"])
    reg = NearestSamplesRegularizer(sigma=0.5, num_nearest=10, reduction=reduction)
    pts.grad = nrm.grad = None
    ln, lp = reg(idx, dw, pts, nrm)
    (0.5 * ln + 2.0 * lp).backward()
    nearest = ns.nearest(idx, dw.detach().contiguous(), pts.detach().contiguous(), 10).cpu().numpy()
    rn, rp, gp, gn = _regularizer_fp64(nearest, pts.detach().cpu().numpy(), nrm.detach().cpu().numpy(), 0.5)
    N = rn.shape[0]
    s = 1.0 / N if reduction == "mean" else 1.0
    assert (nearest > 0).any() and rn.sum() > 0
    np.testing.assert_allclose(float(ln), rn.sum() * s, rtol=1e-5)
    np.testing.assert_allclose(float(lp), rp.sum() * s, rtol=1e-4, atol=1e-9)
    for got, ref in ((pts.grad, 2.0 * s * gp), (nrm.grad, 0.5 * s * gn)):
        got = got.cpu().numpy()[0].astype(np.float64)
        assert np.linalg.norm(got - ref) <= 1e-5 * np.linalg.norm(ref) + 1e-12
    with pytest.raises(ValueError):
        NearestSamplesRegularizer(reduction="max")(idx, dw, pts, nrm)
