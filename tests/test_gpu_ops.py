"""CUDA ops (through the C ABI) against the CPU oracle: transform, EWA
splatting, depth compositing, interpolation and shading, forward and backward.

Tolerances: operations whose arithmetic is spelled out in the reference's
order with exact-rounding intrinsics are compared bit for bit; the EWA
weight differs only by CUDA's expf (<= 2 ulp), hence 1e-6 relative L2; atomic
gradient sums and the FP32 chain rule against the FP64 oracle use 1e-3.
"""
import numpy as np
import pytest
import torch

import oracle

pytestmark = pytest.mark.gpu

DEV = "cuda:0"


def rel_l2(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-30)


def T(a, dtype=torch.float32):
    return torch.as_tensor(np.ascontiguousarray(a)).to(device=DEV, dtype=dtype)


def scene(rng, B, N, W, H, f, behind=0.05):
    pts = np.zeros((B, N, 3), np.float32)
    nrm = np.zeros((B, N, 3), np.float32)
    for b in range(B):
        z = rng.uniform(-2.4, -1.6, N)
        pts[b, :, 2] = z
        pts[b, :, 0] = rng.uniform(-0.5, 0.5, N) * (-z) * W / f
        pts[b, :, 1] = rng.uniform(-0.5, 0.5, N) * (-z) * H / f
        k = int(behind * N)
        pts[b, :k, 2] *= -1
        n = rng.normal(size=(N, 3))
        n[:, 2] = np.abs(n[:, 2]) + 0.8
        nrm[b] = n / np.linalg.norm(n, axis=1, keepdims=True)
    return pts, nrm


@pytest.fixture(scope="module")
def ops():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from unbiased_differentiable_splatting_gb300 import _lib
    from unbiased_differentiable_splatting_gb300.cudaExtensions import (filtering, interpolation, shading, splatting,
                                                                        transform)
    _lib.load()
    return dict(transform=transform, splatting=splatting, filtering=filtering, interpolation=interpolation,
                shading=shading)


@pytest.mark.parametrize("vb", [1, 3])
def test_transform(ops, vb):
    rng = np.random.default_rng(1)
    B, N = 3, 5000
    M = rng.normal(size=(B, 4, 4)).astype(np.float32)
    M[:, 3] = [0, 0, 0, 1]
    v = rng.normal(size=(vb, N, 3)).astype(np.float32)
    g = rng.normal(size=(B, N, 3)).astype(np.float32)
    tr = ops["transform"]
    for affine in (True, False):
        fwd = tr.affineForward if affine else tr.linearForward
        bwd = tr.affineBackward if affine else tr.linearBackward
        out = fwd(T(M), T(v)).cpu().numpy()
        np.testing.assert_array_equal(out, oracle.transform_forward(M, v, affine))
        gM, gv = bwd(T(g), T(M), T(v))
        rM, rv = oracle.transform_backward(g, M, v, affine)
        np.testing.assert_allclose(gM.cpu().numpy(), rM, rtol=1e-4, atol=1e-3)
        np.testing.assert_allclose(gv.cpu().numpy(), rv, rtol=1e-5, atol=1e-5)


def test_transform_empty(ops):
    M = T(np.eye(4, dtype=np.float32)[None])
    out = ops["transform"].affineForward(M, T(np.zeros((1, 0, 3), np.float32)))
    assert out.shape == (1, 0, 3)


@pytest.mark.parametrize("B,sdb", [(1, 1), (2, 1), (2, 2)])
def test_splatting(ops, B, sdb):
    rng = np.random.default_rng(2 + B + sdb)
    W, H, K, N, f = 40, 32, 6, 400, 35.0
    pts, nrm = scene(rng, B, N, W, H, f, behind=0.0)
    sd = rng.uniform(0.008, 0.03, size=(sdb, N, 2)).astype(np.float32)
    idx = rng.integers(-1, N, size=(B, W, H, K)).astype(np.int32)
    w = ops["splatting"].forward(W, H, f, T(idx, torch.int32), T(pts), T(nrm), T(sd), 0.0).cpu().numpy()
    wr = oracle.splat_forward(W, H, f, idx, pts, nrm, sd, 0.0)
    assert rel_l2(w, wr) < 1e-6
    assert np.all(w[idx < 0] == 0)
    g = rng.normal(size=(B, W, H, K)).astype(np.float32)
    gp, gn, gs = ops["splatting"].backward(W, H, f, T(g), T(idx, torch.int32), T(pts), T(nrm), T(sd), 0.0)
    rp, rn, rs = oracle.splat_backward(W, H, f, g, idx, pts, nrm, sd, 0.0)
    assert rel_l2(gp.cpu().numpy(), rp) < 1e-3
    assert rel_l2(gn.cpu().numpy(), rn) < 1e-3
    assert rel_l2(gs.cpu().numpy(), rs) < 1e-3


def test_splatting_smoothing(ops):
    rng = np.random.default_rng(5)
    W, H, K, N, f = 24, 24, 4, 100, 20.0
    pts, nrm = scene(rng, 1, N, W, H, f, behind=0.0)
    sd = rng.uniform(0.01, 0.03, size=(1, N, 2)).astype(np.float32)
    idx = rng.integers(0, N, size=(1, W, H, K)).astype(np.int32)
    w = ops["splatting"].forward(W, H, f, T(idx, torch.int32), T(pts), T(nrm), T(sd), 0.3).cpu().numpy()
    assert rel_l2(w, oracle.splat_forward(W, H, f, idx, pts, nrm, sd, 0.3)) < 1e-6


@pytest.mark.parametrize("K,pb", [(8, 1), (5, 2), (16, 2), (40, 1)])
def test_filtering(ops, K, pb):
    rng = np.random.default_rng(10 + K)
    B, W, H, N, f = 2, 20, 18, 200, 18.0
    pts, nrm = scene(rng, pb, N, W, H, f)
    idx = rng.integers(-1, N, size=(B, W, H, K)).astype(np.int32)
    w = rng.uniform(0, 1, size=(B, W, H, K)).astype(np.float32)
    w[..., 0] = np.where(rng.uniform(size=(B, W, H)) < 0.2, 1.0, w[..., 0])
    w[..., 1] = np.where(rng.uniform(size=(B, W, H)) < 0.2, 0.0, w[..., 1])
    out = ops["filtering"].forward(T(idx, torch.int32), T(w), W, H, f, T(pts), T(nrm)).cpu().numpy()
    np.testing.assert_array_equal(out, oracle.filter_forward(idx, w, W, H, f, pts, nrm))
    g = rng.normal(size=(B, W, H, K)).astype(np.float32)
    gout = ops["filtering"].backward(T(idx, torch.int32), T(w), T(g), W, H, f, T(pts), T(nrm)).cpu().numpy()
    np.testing.assert_array_equal(gout, oracle.filter_backward(idx, w, g, W, H, f, pts, nrm))


@pytest.mark.parametrize("C,ab", [(3, 1), (8, 2), (20, 1)])
def test_interpolation(ops, C, ab):
    rng = np.random.default_rng(20 + C)
    B, W, H, K, N = 2, 16, 12, 6, 150
    idx = rng.integers(-1, N, size=(B, W, H, K)).astype(np.int32)
    w = rng.uniform(0, 1, size=(B, W, H, K)).astype(np.float32)
    a = rng.normal(size=(ab, N, C)).astype(np.float32)
    out = ops["interpolation"].forward(T(idx, torch.int32), T(w), T(a)).cpu().numpy()
    np.testing.assert_array_equal(out, oracle.interp_forward(idx, w, a))
    g = rng.normal(size=(B, W, H, C)).astype(np.float32)
    gw, ga = ops["interpolation"].backward(T(g), T(idx, torch.int32), T(w), T(a))
    rw, ra = oracle.interp_backward(g, idx, w, a)
    np.testing.assert_array_equal(gw.cpu().numpy(), rw)
    np.testing.assert_allclose(ga.cpu().numpy(), ra, rtol=1e-4, atol=1e-5)


def test_shading(ops):
    rng = np.random.default_rng(30)
    B, W, H, L = 2, 16, 20, 3
    nrm = rng.normal(size=(B, W, H, 3)).astype(np.float32)
    dif = rng.uniform(0, 1, size=(B, W, H, 3)).astype(np.float32)
    dirs = rng.normal(size=(B, L, 3)).astype(np.float32)
    I = rng.uniform(0.3, 2, size=(1, L, 3)).astype(np.float32)
    sh = ops["shading"]
    out = sh.forward(T(dirs), T(I), T(nrm), T(dif)).cpu().numpy()
    np.testing.assert_array_equal(out, oracle.shade_forward(dirs, I, nrm, dif))
    g = rng.normal(size=(B, W, H, 3)).astype(np.float32)
    got = sh.backward(T(g), T(dirs), T(I), T(nrm), T(dif))
    ref = oracle.shade_backward(g, dirs, I, nrm, dif)
    for a, b in zip(got, ref):
        np.testing.assert_allclose(a.cpu().numpy(), b, rtol=1e-4, atol=1e-4)
    coef = rng.uniform(-0.3, 0.3, size=(B, 3, 9)).astype(np.float32)
    out = sh.forwardSh(T(coef), T(nrm), T(dif)).cpu().numpy()
    np.testing.assert_array_equal(out, oracle.shade_sh_forward(coef, nrm, dif))
    got = sh.backwardSh(T(g), T(coef), T(nrm), T(dif))
    ref = oracle.shade_sh_backward(g, coef, nrm, dif)
    for a, b in zip(got, ref):
        np.testing.assert_allclose(a.cpu().numpy(), b, rtol=1e-4, atol=1e-4)


def test_bad_inputs_raise(ops):
    with pytest.raises(ValueError):
        ops["transform"].affineForward(torch.zeros(1, 4, 4), torch.zeros(1, 5, 3))  # CPU tensors
    with pytest.raises(TypeError):
        ops["interpolation"].forward(T(np.zeros((1, 2, 2, 1), np.float32)), T(np.zeros((1, 2, 2, 1), np.float32)),
                                     T(np.zeros((1, 3, 3), np.float32)))  # float indices
    with pytest.raises(ValueError):
        x = T(np.zeros((1, 5, 6), np.float32))[:, :, :3]
        ops["transform"].affineForward(T(np.eye(4, dtype=np.float32)[None]), x)  # non-contiguous
