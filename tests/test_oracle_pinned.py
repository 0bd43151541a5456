"""The CPU oracle against golden fixtures produced by the reference's own
functions (tests/golden/make_golden.py over the reference shim)."""
import numpy as np
import pytest

import oracle


def rel_l2(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-30)


def test_expand_bits(golden):
    g = golden("fgt")
    L = oracle.lib()
    L.orc_expand_bits.restype = oracle.ctypes.c_uint
    mine = np.array([L.orc_expand_bits(oracle.ctypes.c_uint(v)) for v in range(1024)], np.uint32)
    np.testing.assert_array_equal(mine, g["expand_bits"])


def test_ewa_weight_matches_reference(golden):
    g = golden("ewa")
    w = np.zeros_like(g["w"])
    raw = np.zeros_like(g["raw"])
    L = oracle.lib()
    for i in range(len(w)):
        r = np.zeros(1, np.float32)
        w[i] = L.orc_ewa_weight(oracle.P(g["pix"][i]), oracle.F(g["W"]), oracle.F(g["H"]), oracle.F(g["f"]),
                                oracle.P(g["pts"][i]), oracle.P(g["nrm"][i]), oracle.P(g["sd"][i]),
                                oracle.F(g["smoothing"]), oracle.P(r))
        raw[i] = r[0]
    # same float / double operation sequence; libm expf on both sides
    np.testing.assert_array_equal(w, g["w"])
    np.testing.assert_array_equal(raw, g["raw"])


def test_screen_points_match_reference(golden):
    g = golden("ewa")
    s = oracle.to_screenspace(g["W"], g["H"], g["f"], g["pts"])
    np.testing.assert_array_equal(s, g["screen"])


def test_ewa_gradient_matches_reference(golden):
    g = golden("ewa")
    ok = (g["raw"] <= 1.0) & (g["raw"] > 1e-6)
    assert ok.sum() > 50
    errs = []
    for i in np.nonzero(ok)[0]:
        gp, gn, gs = oracle.ewa_grad(g["pix"][i], g["W"], g["H"], g["f"], g["pts"][i], g["nrm"][i], g["sd"][i],
                                     g["smoothing"])
        ref = np.concatenate([g["gp"][i], g["gn"][i], g["gs"][i]]).astype(np.float64)
        mine = np.concatenate([gp, gn, gs])
        errs.append(np.linalg.norm(mine - ref) / (np.linalg.norm(ref) + 1e-12))
    # the reference gradient is float32 through a cancellation-prone Jacobian
    # (it agrees with FP64 finite differences to ~3e-4); the oracle is FP64
    assert np.median(errs) < 1e-4
    assert np.max(errs) < 2e-3


def test_splatting_ops_match_reference(golden):
    g = golden("pixel_ops")
    W, H, f = int(g["W"]), int(g["H"]), float(g["f"])
    w = oracle.splat_forward(W, H, f, g["idx"], g["pts"], g["nrm"], g["sd"], 0.0)
    np.testing.assert_array_equal(w, g["splat_w"])
    gp, gn, gs = oracle.splat_backward(W, H, f, g["splat_gin"], g["idx"], g["pts"], g["nrm"], g["sd"], 0.0)
    assert rel_l2(gp, g["splat_gp"]) < 2e-3
    assert rel_l2(gn, g["splat_gn"]) < 2e-3
    assert rel_l2(gs, g["splat_gs"]) < 2e-3


def test_filtering_matches_reference(golden):
    g = golden("pixel_ops")
    W, H, f = int(g["W"]), int(g["H"]), float(g["f"])
    out = oracle.filter_forward(g["idx"], g["filt_w"], W, H, f, g["pts"], g["nrm"])
    np.testing.assert_array_equal(out, g["filt_out"])
    gout = oracle.filter_backward(g["idx"], g["filt_w"], g["filt_gin"], W, H, f, g["pts"], g["nrm"])
    np.testing.assert_array_equal(gout, g["filt_gout"])


def test_shading_matches_reference(golden):
    g = golden("shading")
    out = oracle.shade_forward(g["dirs"], g["I"], g["nrm"], g["dif"])
    np.testing.assert_array_equal(out, g["out"])
    gd, gI, gn, gdf = oracle.shade_backward(g["gin"], g["dirs"], g["I"], g["nrm"], g["dif"])
    assert rel_l2(gd, g["gdirs"]) < 1e-5
    assert rel_l2(gI, g["gI"]) < 1e-5
    np.testing.assert_allclose(gn, g["gn"], rtol=1e-5, atol=1e-6)
    np.testing.assert_allclose(gdf, g["gdif"], rtol=1e-5, atol=1e-6)


def test_sh_shading_matches_reference(golden):
    g = golden("shading")
    sh = oracle.shade_sh_forward(g["coef"], g["nrm"], g["dif"])
    np.testing.assert_array_equal(sh, g["sh"])
    gc, gn, gd = oracle.shade_sh_backward(g["gin"], g["coef"], g["nrm"], g["dif"])
    assert rel_l2(gc, g["sh_gc"]) < 1e-5
    np.testing.assert_allclose(gn, g["sh_gn"], rtol=1e-4, atol=1e-6)
    np.testing.assert_allclose(gd, g["sh_gd"], rtol=1e-6, atol=1e-7)


def test_transform_matches_reference(golden):
    g = golden("transform")
    for name, affine in (("affine", True), ("linear", False)):
        out = oracle.transform_forward(g["M"], g["v"], affine)
        np.testing.assert_array_equal(out, g[f"{name}_out"])
        gM, gv = oracle.transform_backward(g[f"{name}_gin"], g["M"], g["v"], affine)
        np.testing.assert_allclose(gM, g[f"{name}_gM"], rtol=1e-4, atol=1e-4)
        np.testing.assert_allclose(gv, g[f"{name}_gv"], rtol=1e-4, atol=1e-5)


def test_karras_topology_matches_reference(golden):
    g = golden("karras")
    keys = g["keys32"]
    n = len(keys)
    # a tiny scene is not needed: drive the oracle's hierarchy through a tree
    # whose keys are given, by building screen points that produce them is
    # awkward, so compare through the exported C helper on synthetic keys
    left = np.zeros(n - 1, np.int32)
    right = np.zeros(n - 1, np.int32)
    lib = oracle.lib()
    lib.orc_karras_from_keys(oracle.C(n), oracle.P(np.ascontiguousarray(keys, np.uint32)), oracle.P(left),
                             oracle.P(right))
    np.testing.assert_array_equal(left, g["left"])
    np.testing.assert_array_equal(right, g["right"])


def test_hermite_pieces_match_reference(golden):
    g = golden("fgt")
    L = oracle.lib()
    herm = np.zeros_like(g["herm"])
    for i, t in enumerate(g["ts"]):
        L.orc_hermite_function(oracle.F(t), oracle.C(16), oracle.C(oracle.LIBM), oracle.P(herm[i]))
    np.testing.assert_array_equal(herm, g["herm"])
    L.orc_hermite_error.restype = oracle.F
    herr = np.array([L.orc_hermite_error(oracle.F(r), oracle.F(n), oracle.C(int(d)), oracle.C(oracle.LIBM))
                     for r, n, d in zip(g["rs"], g["nrs"], g["degs"])], np.float32)
    np.testing.assert_array_equal(herr, g["herr"])


@pytest.mark.parametrize("name", ["s1", "s2", "s3"])
def test_sampler_matches_reference(golden, name):
    g = {k[len(name) + 1:]: v for k, v in golden("sampler").items() if k.startswith(name + "_")}
    W, H, K = int(g["W"]), int(g["H"]), int(g["K"])
    # the reference's per-pixel hash map holds K*depth entries; it overflows
    # for K = 1, where the single round never reads it back, so the samples
    # are still defined.  Elsewhere the fixtures must not overflow.
    if oracle.num_rounds(K) > 1:
        assert int(g["overflows"]) == 0
    t = oracle.Tree(W, H, float(g["f"]), g["pts"], float(g["h"]), float(g["radius"]), float(g["precision"]),
                    flavour=oracle.LIBM)
    assert t.n == int(g["n_visible"])
    e = t.export()
    np.testing.assert_array_equal(e["keys"], g["keys"])
    np.testing.assert_array_equal(e["ids"], g["ids"])
    np.testing.assert_array_equal(e["left"][: t.n - 1], g["left"][: t.n - 1])
    np.testing.assert_array_equal(e["right"][: t.n - 1], g["right"][: t.n - 1])
    np.testing.assert_array_equal(e["degree"], g["degree"])
    np.testing.assert_array_equal(e["centre"], g["centre"])
    R = oracle.num_rounds(K)
    uni = g["uniforms"].reshape(W * H, R, K)
    idx = t.sample(W, H, K, float(g["precision"]), uniforms=uni, flavour=oracle.LIBM)
    np.testing.assert_array_equal(idx, g["indices"])
