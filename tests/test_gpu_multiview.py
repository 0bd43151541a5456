"""Views of different sizes in one sampling call (one descent launch over
all views' pixels) against the CPU oracle view by view, and the multi-view
renderer built on it."""
import numpy as np
import pytest
import torch

import oracle

pytestmark = pytest.mark.gpu
DEV = "cuda:0"


@pytest.fixture(scope="module")
def smp():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from unbiased_differentiable_splatting_gb300 import _lib, library  # noqa: F401  (torch.ops.uds)
    from unbiased_differentiable_splatting_gb300.cudaExtensions import sampling
    _lib.load()
    return sampling


def _views_scene(rng, N, views):
    P, Nn = [], []
    for (W, H, f) in views:
        z = rng.uniform(-2.4, -1.6, N)
        p = np.stack([rng.uniform(-0.5, 0.5, N) * (-z) * W / f, rng.uniform(-0.5, 0.5, N) * (-z) * H / f, z], 1)
        n = rng.normal(size=(N, 3))
        n[:, 2] = np.abs(n[:, 2]) + 0.5
        n /= np.linalg.norm(n, axis=1, keepdims=True)
        P.append(p)
        Nn.append(n)
    sd = rng.uniform(0.005, 0.012, size=(1, N, 2))
    return np.stack(P).astype(np.float32), np.stack(Nn).astype(np.float32), sd.astype(np.float32)


@pytest.mark.parametrize("K", [8, 13])
def test_sample_views_matches_oracle(smp, K):
    rng = np.random.default_rng(3 + K)
    views = [(48, 40, 40.0), (32, 32, 30.0), (64, 24, 50.0), (32, 32, 30.0)]
    pts, nrm, sd = _views_scene(rng, 1500, views)
    T = lambda a: torch.as_tensor(a).to(DEV)  # noqa: E731
    out, st = smp.sample_views(views, T(pts), T(nrm), None, T(sd), K, 0.0, 0.01, seed=77, return_stats=True)
    assert len(out) == len(views)
    for b, (W, H, f) in enumerate(views):
        assert tuple(out[b].shape) == (1, W, H, K)
        ref, rst = oracle.sample_view(W, H, f, pts[b], nrm[b], sd[0], K, 0.0, 0.01, h=float(st["h"][b]), seed=77,
                                      view=b)
        assert int(st["n_visible"][b]) == rst["n_visible"]
        np.testing.assert_array_equal(out[b].cpu().numpy()[0], ref)
    # the registered op gives the same indices
    res = torch.ops.uds.sample_views([v[0] for v in views], [v[1] for v in views], [v[2] for v in views], T(pts),
                                     T(nrm), T(sd), K, 0.0, 0.01, 77, None)
    for a, b in zip(res, out):
        assert torch.equal(a, b)
    # every tile shape and both ways of sharing out the child masses agree
    for tx, sp in ((4, 1), (16, 0), (32, 1)):
        alt = smp.sample_views(views, T(pts), T(nrm), None, T(sd), K, 0.0, 0.01, seed=77, tile_x=tx, spread=sp)
        for a, b in zip(alt, out):
            assert torch.equal(a, b), (tx, sp)


def test_tune_views_caches_batch_choice(smp, tmp_path, monkeypatch):
    from unbiased_differentiable_splatting_gb300 import autotune
    monkeypatch.setenv("UDS_AUTOTUNE_CACHE", str(tmp_path / "cache.json"))
    autotune.reset()
    rng = np.random.default_rng(9)
    views = [(48, 40, 40.0), (32, 32, 30.0)]
    pts, nrm, sd = _views_scene(rng, 1500, views)
    T = lambda a: torch.as_tensor(a).to(DEV)  # noqa: E731
    best, times = autotune.tune_views(views, T(pts), T(nrm), T(sd), 8, 0.0, 0.01, reps=1, candidates=(8, 16))
    assert len(times) == 2 * len(autotune.SPREADS)
    assert autotune.lookup_views(torch.cuda.get_device_name(0), views, pts.shape[1], 8) == best
    autotune.reset()


def test_multiview_renderer(smp):
    """MultiViewSplatting: its indices are the sampler's, each view's image
    is the fused render pass of its view, and gradients reach the splats and
    the poses of every view."""
    from unbiased_differentiable_splatting_gb300 import scenes
    from unbiased_differentiable_splatting_gb300.render import MultiViewSplatting, RenderOptions
    sc = scenes.harmonic_scene(n=5000, sd_range=(0.01, 0.02), width=64, seed=2)
    cp, co = scenes.orbit_cameras(5, distance=2.0, seed=0)
    ld, li, amb = scenes._lights(5)
    f64, f32 = scenes.focal_from_fov(64), scenes.focal_from_fov(32)
    views = [(64, 64, f64), (64, 64, f64), (32, 32, f32), (32, 32, f32), (64, 48, f64)]
    r = MultiViewSplatting(RenderOptions(numSamples=8, precision=0.01, shadingMode="forward"), None, views, 0.1,
                           100.0, 0.0).to(DEV)
    assert [g[:2] for g in r.groups] == [(0, 2), (2, 2), (4, 1)]
    r.sample_kwargs = {"seed": 5}
    d = {k: v.to(DEV) for k, v in sc.items() if isinstance(v, torch.Tensor)}
    pos, quat = cp.to(DEV).requires_grad_(True), co.to(DEV).requires_grad_(True)
    pts = d["points"].clone().requires_grad_(True)
    imgs, idxs, dws = r(pos, quat, pts, d["normals"], d["stddevs"], d["colors"], amb.to(DEV), ld.to(DEV),
                        li.to(DEV))
    assert [tuple(i.shape) for i in imgs] == [(1, w, h, 3) for (w, h, _) in views]
    assert all((i >= 0).any() for i in idxs)
    sum((im ** 2).sum() for im in imgs).backward()
    assert torch.isfinite(pts.grad).all() and pts.grad.abs().sum() > 0
    assert (quat.grad.abs().sum(1) > 0).all() and (pos.grad.abs().sum(1) > 0).all()
    with pytest.raises(ValueError):
        MultiViewSplatting(RenderOptions(shadingMode="deferred"), None, views, 0.1, 100.0, 0.0)
