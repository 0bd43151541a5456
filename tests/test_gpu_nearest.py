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


def test_regularizer_on_render(ns):
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
    reg = NearestSamplesRegularizer(sigma=0.5, num_nearest=10)
    ln, lp = reg(idx, dw, pts, nrm)
    (ln + lp).backward()
    assert torch.isfinite(ln) and torch.isfinite(lp) and float(ln.detach()) > 0
    assert torch.isfinite(pts.grad).all() and pts.grad.abs().sum() > 0
