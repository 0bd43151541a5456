"""pixelgather.scatter / gather on the GPU against the oracle."""
import numpy as np
import pytest
import torch

import oracle

pytestmark = pytest.mark.gpu
DEV = "cuda:0"


@pytest.fixture(scope="module")
def pg():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from unbiased_differentiable_splatting_gb300.cudaExtensions import pixelgather
    return pixelgather


def case(seed, B=2, W=33, H=27, K=8, N=500, C=3, hot=False):
    rng = np.random.default_rng(seed)
    idx = rng.integers(-1, N, size=(B, W, H, K)).astype(np.int32)
    if hot:  # heavy contention: most samples on a few splats
        idx[rng.random(idx.shape) < 0.7] = rng.integers(0, 4)
    v = rng.normal(size=(B, N, C)).astype(np.float32)
    g = rng.normal(size=(B, W, H, K, C)).astype(np.float32)
    return idx, v, g, N


@pytest.mark.parametrize("hot", [False, True])
def test_scatter_gather(pg, hot):
    idx, v, g, N = case(1, hot=hot)
    ti = torch.as_tensor(idx).to(DEV)
    s = pg.scatter(ti, torch.as_tensor(v).to(DEV))
    np.testing.assert_array_equal(s.cpu().numpy(), oracle.pixel_scatter(idx, v))
    ref = oracle.pixel_gather(idx, g, N)
    tg = torch.as_tensor(g).to(DEV)
    det = pg.gather(ti, tg, N, deterministic=True).cpu().numpy()
    np.testing.assert_array_equal(det, ref)  # same additions in the same order
    det2 = pg.gather(ti, tg, N, deterministic=True).cpu().numpy()
    np.testing.assert_array_equal(det2, det)
    at = pg.gather(ti, tg, N).cpu().numpy()
    np.testing.assert_allclose(at, ref, rtol=1e-4, atol=1e-4)


@pytest.mark.parametrize("B,W,H,K,N,hot", [(1, 512, 512, 8, 300_000, True), (3, 128, 96, 5, 5_000_000, False),
                                            (1, 7, 5, 1, 1, False)])
def test_deterministic_gather_large(pg, B, W, H, K, N, hot):
    """Bit-exact against the oracle's sequential sums at sizes that take up to
    three radix passes, with one splat holding about 70% of 2M samples."""
    idx, _, g, _ = case(3, B=B, W=W, H=H, K=K, N=N, C=2, hot=hot)
    ref = oracle.pixel_gather(idx, g, N)
    ti, tg = torch.as_tensor(idx).to(DEV), torch.as_tensor(g).to(DEV)
    det = pg.gather(ti, tg, N, deterministic=True).cpu().numpy()
    np.testing.assert_array_equal(det, ref)


def test_pixel_scatter_gather_autograd(pg):
    from unbiased_differentiable_splatting_gb300.extensions import PixelScatterGather
    idx, v, g, N = case(2, B=1, W=16, H=16, K=4, N=60, C=2)
    ti = torch.as_tensor(idx).to(DEV)
    tv = torch.as_tensor(v).to(DEV).requires_grad_(True)
    out = PixelScatterGather.apply(ti, tv)
    (out * torch.as_tensor(g).to(DEV)).sum().backward()
    np.testing.assert_allclose(tv.grad.cpu().numpy(), oracle.pixel_gather(idx, g, N), rtol=1e-4, atol=1e-5)
