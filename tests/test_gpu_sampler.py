"""FMM tree and sampler on the GPU (through the C ABI) against the CPU oracle.

Bit-exact: Morton keys, splat order, tree topology, Hermite degrees, node
centres and boxes, FGT node masses, sampled indices (given the same uniforms
and the bandwidth the op reports).  FGT masses against the FP64 direct Gauss
sum: within the truncation bound `precision` (absolute) plus 1e-4 relative.
"""
import numpy as np
import pytest
import torch

import oracle

pytestmark = pytest.mark.gpu
DEV = "cuda:0"


def T(a, dtype=torch.float32):
    return torch.as_tensor(np.ascontiguousarray(a)).to(device=DEV, dtype=dtype)


@pytest.fixture(scope="module")
def smp():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from unbiased_differentiable_splatting_gb300 import _lib
    from unbiased_differentiable_splatting_gb300.cudaExtensions import sampling
    _lib.load()
    return sampling


def camera_scene(rng, N, W, H, f, sd=(0.004, 0.012), behind=0.05, offscreen=0.05, dup=0.02):
    z = rng.uniform(-2.4, -1.6, N)
    pts = np.stack([rng.uniform(-0.5, 0.5, N) * (-z) * W / f, rng.uniform(-0.5, 0.5, N) * (-z) * H / f, z], 1)
    k1, k2 = int(behind * N), int((behind + offscreen) * N)
    pts[:k1, 2] *= -1
    pts[k1:k2, 0] *= 5
    nd = int(dup * N)
    if nd:
        pts[-nd:] = pts[k2:k2 + nd]  # coincident splats -> equal Morton keys
    n = rng.normal(size=(N, 3))
    n[:, 2] = np.abs(n[:, 2]) + 0.5
    n /= np.linalg.norm(n, axis=1, keepdims=True)
    s = rng.uniform(sd[0], sd[1], size=(N, 2))
    return pts.astype(np.float32), n.astype(np.float32), s.astype(np.float32)


def sphere_cam(n=4096, W=128, seed=0):
    from unbiased_differentiable_splatting_gb300 import scenes
    sc = scenes.sphere_scene(n=n, width=W, seed=seed)
    pts, nrm = scenes.camera_space(sc)
    facing = nrm[..., 2:] > 0
    nrm = torch.where(facing, -nrm, nrm)  # BackfaceCulling
    return pts.numpy()[0], nrm.numpy()[0], sc["stddevs"].numpy()[0], sc["focal"], W


@pytest.mark.parametrize("seed", [0, 1])
def test_tree_bit_exact(smp, seed):
    rng = np.random.default_rng(seed)
    W, H, f, N = 96, 80, 80.0, 3000
    pts, nrm, sd = camera_scene(rng, N, W, H, f)
    tree = smp.build_tree(W, H, f, T(pts[None]), T(nrm[None]), T(sd[None]), 8, 0.0, 0.01)
    h_ref = oracle.view_bandwidth(W, H, f, pts, nrm, sd, 0.0)
    assert tree["h"] == np.float32(h_ref)
    r_ref = oracle.cull_radius(tree["h"], 0.01)
    assert tree["radius"] == np.float32(r_ref)
    t = oracle.Tree(W, H, f, pts, tree["h"], tree["radius"], 0.01)
    assert tree["n_visible"] == t.n
    e = t.export()
    n = t.n
    np.testing.assert_array_equal(tree["keys"].numpy().view(np.uint32), e["keys"])
    np.testing.assert_array_equal(tree["ids"].numpy(), e["ids"])
    np.testing.assert_array_equal(tree["left"].numpy()[: n - 1], e["left"][: n - 1])
    np.testing.assert_array_equal(tree["right"].numpy()[: n - 1], e["right"][: n - 1])
    np.testing.assert_array_equal(tree["parent"].numpy(), e["parent"])
    np.testing.assert_array_equal(tree["count"].numpy(), e["count"])
    np.testing.assert_array_equal(tree["degree"].numpy(), e["degree"])
    np.testing.assert_array_equal(tree["centre"].numpy(), e["centre"])
    np.testing.assert_array_equal(tree["box"].numpy(), e["box"])
    assert tree["n_coefs"] == t.num_coefs


def test_fgt_masses(smp):
    rng = np.random.default_rng(3)
    W, H, f, N = 64, 64, 55.0, 2500
    pts, nrm, sd = camera_scene(rng, N, W, H, f, sd=(0.01, 0.03), behind=0, offscreen=0, dup=0)
    for precision in (0.01, 1e-4):
        tree = smp.build_tree(W, H, f, T(pts[None]), T(nrm[None]), T(sd[None]), 8, 0.0, precision)
        t = oracle.Tree(W, H, f, pts, tree["h"], tree["radius"], precision)
        n = t.n
        M = 2 * n - 1
        nodes = rng.integers(0, M, size=600).astype(np.int32)
        nodes[:40] = 0
        q = rng.uniform(0, W, size=(600, 2)).astype(np.float32)
        got = smp.fgt_eval(tree, T(nodes, torch.int32), T(q)).cpu().numpy()
        ref = np.array([t.node_weight(int(v), q[i]) for i, v in enumerate(nodes)], np.float32)
        np.testing.assert_array_equal(got, ref)
        direct = np.array([t.direct_weight(int(v), q[i].astype(np.float64)) for i, v in enumerate(nodes)])
        err = np.abs(got - direct)
        # truncation drops sources below precision / count each (<= precision
        # in total); the Hermite series adds at most `precision` per node
        assert np.all(err <= 3 * precision + 1e-4 * direct), (precision, err.max())


def _sample_both(smp, pts, nrm, sd, W, H, f, K, precision=0.01, uniforms=None, seed=11):
    B = pts.shape[0]
    kw = dict(seed=seed, return_stats=True)
    if uniforms is not None:
        kw["uniforms"] = T(uniforms)
    idx, st = smp.sample(W, H, f, T(pts), T(nrm), T(np.zeros_like(pts)), T(sd), K, 0.0, precision, **kw)
    got = idx.cpu().numpy()
    R = oracle.num_rounds(K)
    for b in range(B):
        h = float(st["h"][b])
        u = None if uniforms is None else uniforms[b].reshape(W * H, R, K)
        ref, rst = oracle.sample_view(W, H, f, pts[b], nrm[b], sd[min(b, sd.shape[0] - 1)], K, 0.0, precision, h=h,
                                      uniforms=u, seed=seed, view=b)
        assert int(st["n_visible"][b]) == rst["n_visible"]
        assert float(st["radius"][b]) == np.float32(rst["radius"])
        diff = (got[b] != ref).any(-1)
        assert not diff.any(), f"view {b}: {diff.sum()} pixels differ, first at {np.argwhere(diff)[:3].tolist()}"
    return got, st


@pytest.mark.parametrize("K", [1, 4, 8, 13])
def test_sample_bit_exact_uniforms(smp, K):
    rng = np.random.default_rng(40 + K)
    W, H, f, N = 48, 40, 40.0, 1500
    pts, nrm, sd = camera_scene(rng, N, W, H, f)
    R = oracle.num_rounds(K)
    u = rng.uniform(2.0 ** -24, 1.0, size=(1, W, H, R, K)).astype(np.float32)
    got, st = _sample_both(smp, pts[None], nrm[None], sd[None], W, H, f, K, uniforms=u)
    assert (got >= 0).any()


def test_sample_bit_exact_philox_multiview(smp):
    rng = np.random.default_rng(50)
    B, W, H, f, N, K = 3, 40, 36, 36.0, 1200, 8
    P, Nn = [], []
    for b in range(B):
        p, n, s = camera_scene(rng, N, W, H, f)
        P.append(p)
        Nn.append(n)
    sd = rng.uniform(0.005, 0.012, size=(1, N, 2)).astype(np.float32)
    _sample_both(smp, np.stack(P), np.stack(Nn), sd, W, H, f, K, seed=123456789)


def test_sample_sphere_128(smp):
    pts, nrm, sd, f, W = sphere_cam()
    got, st = _sample_both(smp, pts[None], nrm[None], sd[None], W, W, f, 8, seed=5)
    assert int(st["n_visible"][0]) == 4096
    assert (got >= 0).mean() > 0.1


def test_sample_edge_cases(smp):
    rng = np.random.default_rng(60)
    W, H, f = 16, 12, 14.0
    # single visible splat
    pts, nrm, sd = camera_scene(rng, 1, W, H, f, behind=0, offscreen=0, dup=0)
    got, st = _sample_both(smp, pts[None], nrm[None], sd[None], W, H, f, 4)
    assert int(st["n_visible"][0]) == 1
    # everything behind the camera: no samples at all
    pts, nrm, sd = camera_scene(rng, 50, W, H, f, behind=1.0, offscreen=0, dup=0)
    got, st = _sample_both(smp, pts[None], nrm[None], sd[None], W, H, f, 4)
    assert int(st["n_visible"][0]) == 0 and np.all(got == -1)
    # no splats
    idx = smp.sample(W, H, f, T(np.zeros((1, 0, 3), np.float32)), T(np.zeros((1, 0, 3), np.float32)),
                     T(np.zeros((1, 0, 3), np.float32)), T(np.zeros((1, 0, 2), np.float32)), 4, 0.0, 0.01)
    assert torch.all(idx == -1)
    # all splats at one point (all Morton keys equal)
    pts, nrm, sd = camera_scene(rng, 40, W, H, f, behind=0, offscreen=0, dup=0)
    pts[:] = pts[0]
    _sample_both(smp, pts[None], nrm[None], sd[None], W, H, f, 8)


@pytest.mark.parametrize("L,K", [(16, 8), (32, 8), (64, 4), (24, 13)])
def test_sample_leaf_size_bit_exact(smp, L, K):
    """Leaf buckets: each round stops at the first node holding <= L splats
    and order-samples over all of them.  Indices equal the oracle's rule,
    with a (B,W,H,R,L) uniforms tensor and with Philox uniforms, in the
    one-view and the uneven multi-view launch; L <= K is the default rule."""
    rng = np.random.default_rng(90 + L + K)
    W, H, f, N = 48, 40, 40.0, 3000
    pts, nrm, sd = camera_scene(rng, N, W, H, f, sd=(0.01, 0.03))
    R, M = oracle.num_rounds(K), max(K, L)
    u = rng.uniform(2.0 ** -24, 1.0, size=(1, W, H, R, M)).astype(np.float32)
    args = (W, H, f, T(pts[None]), T(nrm[None]), T(np.zeros((1, N, 3))), T(sd[None]), K, 0.0, 0.01)
    for kw in (dict(uniforms=T(u)), dict(seed=77)):
        idx, st = smp.sample(*args, leaf_size=L, return_stats=True, **kw)
        h = float(st["h"][0])
        tree = oracle.Tree(W, H, f, pts, h, oracle.cull_radius(h, 0.01), 0.01)
        ref = tree.sample(W, H, K, 0.01, uniforms=u[0].reshape(W * H, R, M) if "uniforms" in kw else None,
                          seed=kw.get("seed", 0), leaf_size=L)
        got = idx.cpu().numpy()[0]
        assert (got >= 0).any()
        np.testing.assert_array_equal(got, ref)
    # the same rule in the uneven launch: view 1 is a smaller view of the same splats
    if K <= 8:
        views = [(W, H, f), (32, 24, 0.6 * f)]
        out = smp.sample_views(views, T(np.stack([pts, pts])), T(np.stack([nrm, nrm])), None, T(sd[None]), K, 0.0,
                               0.01, seed=78, leaf_size=L, return_stats=True)
        for b, (w_, h_, f_) in enumerate(views):
            hb = float(out[1]["h"][b])
            tree = oracle.Tree(w_, h_, f_, pts, hb, oracle.cull_radius(hb, 0.01), 0.01)
            np.testing.assert_array_equal(out[0][b].cpu().numpy()[0],
                                          tree.sample(w_, h_, K, 0.01, seed=78, view=b, leaf_size=L))
    assert torch.equal(smp.sample(*args, seed=5, leaf_size=K), smp.sample(*args, seed=5))


def test_sample_bad_args(smp):
    x = T(np.zeros((1, 4, 3), np.float32))
    s = T(np.zeros((1, 4, 2), np.float32))
    with pytest.raises((RuntimeError, ValueError)):
        smp.sample(8, 8, 8.0, x, x, x, s, 65, 0.0, 0.01)  # K above 64
    with pytest.raises(ValueError):
        smp.sample(8, 8, 8.0, x, x, x, T(np.zeros((2, 4, 2), np.float32)), 4, 0.0, 0.01)
    with pytest.raises((RuntimeError, ValueError)):
        smp.sample(8, 8, 8.0, x, x, x, s, 4, 0.0, 0.01, leaf_size=65)  # leaf size above 64
    with pytest.raises(ValueError):  # uniforms sized for K, not for the leaf size
        smp.sample(8, 8, 8.0, x, x, x, s, 4, 0.0, 0.01, leaf_size=16,
                   uniforms=T(np.full((1, 8, 8, 2, 4), 0.5, np.float32)))


@pytest.mark.parametrize("K", [1, 8, 24])
def test_stochastic_bit_exact(smp, K):
    """Stochastic mode: indices and path probabilities equal the oracle's."""
    rng = np.random.default_rng(70 + K)
    B, W, H, f, N = 2, 40, 36, 36.0, 1500
    P, Nn = [], []
    for b in range(B):
        p, n, s = camera_scene(rng, N, W, H, f)
        P.append(p)
        Nn.append(n)
    sd = rng.uniform(0.005, 0.012, size=(1, N, 2)).astype(np.float32)
    pts, nrm = np.stack(P), np.stack(Nn)
    idx, prob, st = smp.sample_stochastic(W, H, f, T(pts), T(nrm), T(sd), K, 0.0, 0.01, seed=99, return_stats=True)
    idx, prob = idx.cpu().numpy(), prob.cpu().numpy()
    assert int(st["overflow"].sum()) == 0
    for b in range(B):
        ri, rp = oracle.sample_view_stochastic(W, H, f, pts[b], nrm[b], sd[0], K, 0.0, 0.01, h=float(st["h"][b]),
                                               seed=99, view=b)
        np.testing.assert_array_equal(idx[b], ri)
        np.testing.assert_array_equal(prob[b], rp)
    assert (idx >= 0).mean() > 0.3
    assert np.all((prob > 0) == (idx >= 0)) and prob.max() <= 1.0


def test_descent_tile_shapes_agree_and_autotune(smp, tmp_path, monkeypatch):
    """Every warp-tile shape and both ways of sharing out the child masses
    give the same indices; the autotuner times them and caches one."""
    from unbiased_differentiable_splatting_gb300 import autotune
    monkeypatch.setenv("UDS_AUTOTUNE_CACHE", str(tmp_path / "cache.json"))
    autotune.reset()
    rng = np.random.default_rng(80)
    W, H, f, N, K = 72, 56, 60.0, 3000, 8
    pts, nrm, sd = camera_scene(rng, N, W, H, f)
    args = (W, H, f, T(pts[None]), T(nrm[None]), T(np.zeros((1, N, 3))), T(sd[None]), K, 0.0, 0.01)
    ref = smp.sample(*args, seed=3, tile_x=8, spread=0)
    for tx in (4, 8, 16, 32):
        for sp in (0, 1):
            assert torch.equal(smp.sample(*args, seed=3, tile_x=tx, spread=sp), ref), (tx, sp)
    best, times = autotune.tune_descent(W, H, f, T(pts[None]), T(nrm[None]), T(sd[None]), K, 0.0, 0.01)
    assert best["tile_x"] in autotune.CANDIDATES and best["spread"] in autotune.SPREADS
    assert len(times) == len(autotune.CANDIDATES) * len(autotune.SPREADS)
    assert autotune.lookup_config(torch.cuda.get_device_name(0), W, H, N, K) == best
    assert torch.equal(smp.sample(*args, seed=3), ref)  # now with the tuned tile
    autotune.reset()


@pytest.mark.parametrize("P", [4, 6, 8])
def test_fixed_degree_m2m(smp, P):
    """Fixed-degree mode: expansions built by M2M shifts; node masses against
    the FP64 direct Gauss sums, topology unchanged."""
    rng = np.random.default_rng(90 + P)
    W, H, f, N = 64, 56, 60.0, 4000
    precision = 1e-3
    pts, nrm, sd = camera_scene(rng, N, W, H, f, sd=(0.01, 0.03))
    args = (W, H, f, T(pts[None]), T(nrm[None]), T(sd[None]), 8, 0.0, precision)
    ref = smp.build_tree(*args)
    tree = smp.build_tree(*args, fixed_degree=P)
    for k in ("keys", "ids", "left", "right", "parent", "count"):
        assert torch.equal(tree[k], ref[k]), k
    n = tree["n_visible"]
    deg = tree["degree"][: n - 1]
    assert set(deg.unique().tolist()) <= {-1, P} and (deg == P).any()
    assert tree["n_coefs"] == (n - 1) * (P + 1) ** 2
    o = oracle.Tree(W, H, f, pts, tree["h"], oracle.cull_radius(tree["h"], precision), precision)
    nodes = rng.integers(0, 2 * n - 1, 600).astype(np.int32)
    q = rng.uniform(0, W, size=(600, 2)).astype(np.float32)
    got = smp.fgt_eval(tree, T(nodes, torch.int32), T(q)).cpu().numpy()
    direct = np.array([o.direct_weight(int(v), qq.astype(np.float64)) for v, qq in zip(nodes, q)])
    err = np.abs(got - direct)
    assert np.all(err <= 3 * precision + 1e-3 * direct), (P, err.max(), (err / (direct + 1e-9)).max())
    # the sampler runs on the fixed-degree tree and mostly agrees with the adaptive one
    a = smp.sample(W, H, f, T(pts[None]), T(nrm[None]), T(np.zeros((1, N, 3))), T(sd[None]), 8, 0.0, precision,
                   seed=3)
    b = smp.sample(W, H, f, T(pts[None]), T(nrm[None]), T(np.zeros((1, N, 3))), T(sd[None]), 8, 0.0, precision,
                   seed=3, fixed_degree=P)
    assert (a == b).all(-1).float().mean() > 0.9
