"""Generate the golden fixtures of tests/golden/ from the reference itself.

The reference shim oracle/_ref/libudsref.so is compiled (``make -C oracle
ref``, with UDS_REFERENCE_DIR naming the reference checkout) from the
reference's own headers where they lie in that checkout; this script calls
those functions on seeded synthetic inputs and stores inputs and outputs as
compressed .npz files.  It is run by hand where the reference checkout
exists; the fixtures are committed so the tests need neither the reference
nor the shim.

    UDS_REFERENCE_DIR=<checkout> make -C oracle ref
    python tests/golden/make_golden.py
"""
from __future__ import annotations

import ctypes
import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import REF_PATH  # noqa: E402

F32P = ctypes.POINTER(ctypes.c_float)
I32P = ctypes.POINTER(ctypes.c_int)
U32P = ctypes.POINTER(ctypes.c_uint)
U64P = ctypes.POINTER(ctypes.c_ulonglong)
C, F = ctypes.c_int, ctypes.c_float


def P(a):
    if a is None:
        return None
    return a.ctypes.data_as({np.float32: F32P, np.int32: I32P, np.uint32: U32P, np.uint64: U64P}[a.dtype.type])


def f32(a):
    return np.ascontiguousarray(a, np.float32)


def load():
    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "ref"], check=True)
    L = ctypes.CDLL(REF_PATH)
    L.ref_hermite_error.restype = ctypes.c_float
    L.ref_hermite_error.argtypes = [F, F, F]
    L.ref_evaluate_hermite.restype = ctypes.c_float
    L.ref_expand_bits.restype = ctypes.c_uint
    L.ref_expand_bits.argtypes = [ctypes.c_uint]
    L.ref_sample_view.restype = ctypes.c_int
    return L


def scene_small(rng, n, W, H, f, spread=0.45, z=(-2.3, -1.7), hidden=0.1):
    """Random camera-space surfels in front of the camera, normals facing it
    within 60 degrees, a fraction behind the camera or off screen."""
    pts = np.zeros((n, 3))
    pts[:, 2] = rng.uniform(z[0], z[1], n)
    pts[:, 0] = rng.uniform(-spread, spread, n) * -pts[:, 2] / 2.0 * (W / f) * 2.0
    pts[:, 1] = rng.uniform(-spread, spread, n) * -pts[:, 2] / 2.0 * (H / f) * 2.0
    k = int(hidden * n)
    pts[:k // 2, 2] *= -1.0  # behind the camera
    pts[k // 2:k, 0] *= 4.0  # off screen
    nrm = rng.normal(size=(n, 3))
    nrm[:, 2] = np.abs(nrm[:, 2]) + 1.0
    nrm /= np.linalg.norm(nrm, axis=1, keepdims=True)
    return f32(pts), f32(nrm)


def gen_ewa(L, rng):
    W, H, f, sm = 64.0, 48.0, 55.4, 0.0
    n = 400
    pts, nrm = scene_small(rng, n, W, H, f, hidden=0.0)
    sd = f32(rng.uniform(0.004, 0.02, size=(n, 2)))
    sp = np.zeros((n, 2), np.float32)
    L.ref_to_screenspace(C(n), F(W), F(H), F(f), P(pts), P(sp))
    pix = f32(np.round(sp) + rng.integers(-3, 4, size=(n, 2)))
    w = np.zeros(n, np.float32)
    raw = np.zeros(n, np.float32)
    L.ref_ewa_pairs(C(n), P(pix), F(W), F(H), F(f), P(pts), P(nrm), P(sd), F(sm), P(w), P(raw))
    gp, gn, gs = np.zeros((n, 3), np.float32), np.zeros((n, 3), np.float32), np.zeros((n, 2), np.float32)
    L.ref_ewa_grad_pairs(C(n), P(pix), F(W), F(H), F(f), P(pts), P(nrm), P(sd), F(sm), P(gp), P(gn), P(gs))
    return dict(W=W, H=H, f=f, smoothing=sm, pts=pts, nrm=nrm, sd=sd, pix=pix, screen=sp, w=w, raw=raw, gp=gp, gn=gn,
                gs=gs)


def gen_pixel_ops(L, rng):
    B, W, H, K, N = 2, 12, 10, 5, 60
    f = 12.0
    pts = np.zeros((B, N, 3), np.float32)
    nrm = np.zeros((B, N, 3), np.float32)
    for b in range(B):
        pts[b], nrm[b] = scene_small(rng, N, W, H, f, hidden=0.0)
    sd = f32(rng.uniform(0.01, 0.05, size=(1, N, 2)))
    idx = rng.integers(-1, N, size=(B, W, H, K)).astype(np.int32)
    w = np.zeros((B, W, H, K), np.float32)
    L.ref_splat_forward(C(B), C(W), C(H), C(K), F(f), P(idx), P(pts), P(nrm), P(sd), C(1), C(N), F(0.0), P(w))
    gin = f32(rng.normal(size=(B, W, H, K)))
    gp, gn, gs = np.zeros_like(pts), np.zeros_like(nrm), np.zeros_like(sd)
    L.ref_splat_backward(C(B), C(W), C(H), C(K), F(f), P(gin), P(idx), P(pts), P(nrm), P(sd), C(1), C(N), F(0.0),
                         P(gp), P(gn), P(gs))
    # compositing on random weights in [0,1] including exact 0 and 1
    wc = f32(rng.uniform(0, 1, size=(B, W, H, K)))
    wc[..., 0] = np.where(rng.uniform(size=(B, W, H)) < 0.2, 1.0, wc[..., 0])
    wc[..., 1] = np.where(rng.uniform(size=(B, W, H)) < 0.2, 0.0, wc[..., 1])
    fo = np.zeros_like(wc)
    L.ref_filter_forward(C(B), C(W), C(H), C(K), P(idx), P(wc), F(f), C(B), C(N), P(pts), P(nrm), P(fo))
    fg = f32(rng.normal(size=(B, W, H, K)))
    fb = np.zeros_like(wc)
    L.ref_filter_backward(C(B), C(W), C(H), C(K), P(idx), P(wc), P(fg), F(f), C(B), C(N), P(pts), P(nrm), P(fb))
    return dict(B=B, W=W, H=H, K=K, N=N, f=f, pts=pts, nrm=nrm, sd=sd, idx=idx, splat_w=w, splat_gin=gin, splat_gp=gp,
                splat_gn=gn, splat_gs=gs, filt_w=wc, filt_out=fo, filt_gin=fg, filt_gout=fb)


def gen_shading(L, rng):
    B, Pn, Ln = 2, 300, 3
    nrm = rng.normal(size=(B, Pn, 3))
    nrm /= np.linalg.norm(nrm, axis=-1, keepdims=True)
    nrm = f32(nrm * rng.uniform(0.5, 1.5, size=(B, Pn, 1)))
    nrm[0, 0] = 0.0  # degenerate normal
    dif = f32(rng.uniform(0, 1, size=(B, Pn, 3)))
    dirs = rng.normal(size=(B, Ln, 3))
    dirs = f32(dirs / np.linalg.norm(dirs, axis=-1, keepdims=True))
    I = f32(rng.uniform(0.2, 2.0, size=(1, Ln, 3)))
    out = np.zeros_like(nrm)
    L.ref_shade_forward(C(B * Pn), C(Ln), C(B), P(dirs), P(I), C(1), P(nrm), P(dif), P(out))
    gin = f32(rng.normal(size=(B, Pn, 3)))
    gd, gI, gn, gdf = np.zeros_like(dirs), np.zeros_like(I), np.zeros_like(nrm), np.zeros_like(dif)
    L.ref_shade_backward(C(B * Pn), C(Ln), C(B), P(gin), P(dirs), P(I), C(1), P(nrm), P(dif), P(gd), P(gI), P(gn),
                         P(gdf))
    coef = f32(rng.uniform(-0.3, 0.3, size=(B, 3, 9)))
    coef[..., 0] += 0.5
    sh = np.zeros_like(nrm)
    L.ref_shade_sh_forward(C(B * Pn), C(B), P(coef), C(B), P(nrm), P(dif), P(sh))
    gc, gn2, gd2 = np.zeros_like(coef), np.zeros_like(nrm), np.zeros_like(dif)
    L.ref_shade_sh_backward(C(B * Pn), C(B), P(gin), P(coef), C(B), P(nrm), P(dif), P(gc), P(gn2), P(gd2))
    return dict(nrm=nrm, dif=dif, dirs=dirs, I=I, out=out, gin=gin, gdirs=gd, gI=gI, gn=gn, gdif=gdf, coef=coef,
                sh=sh, sh_gc=gc, sh_gn=gn2, sh_gd=gd2)


def gen_transform(L, rng):
    B, N = 3, 200
    M = f32(rng.normal(size=(B, 4, 4)))
    M[:, 3] = [0, 0, 0, 1]
    v = f32(rng.normal(size=(1, N, 3)))
    out = {}
    for mode, name in ((1, "affine"), (0, "linear")):
        o = np.zeros((B, N, 3), np.float32)
        L.ref_transform_forward(C(mode), C(B), P(M), C(1), C(N), P(v), P(o))
        g = f32(rng.normal(size=(B, N, 3)))
        gM, gv = np.zeros_like(M), np.zeros_like(v)
        L.ref_transform_backward(C(mode), C(B), P(g), P(M), C(1), C(N), P(v), P(gM), P(gv))
        out.update({f"{name}_out": o, f"{name}_gin": g, f"{name}_gM": gM, f"{name}_gv": gv})
    return dict(M=M, v=v, **out)


def gen_fgt(L, rng):
    ts = f32(rng.uniform(-3, 3, size=64))
    herm = np.zeros((64, 17), np.float32)
    for i, t in enumerate(ts):
        buf = np.zeros(17, np.float32)
        L.ref_hermite_function(F(t), C(16), P(buf))
        herm[i] = buf
    rs = f32(rng.uniform(0, 1.2, size=50))
    nrs = f32(rng.integers(2, 500, size=50))
    degs = rng.integers(0, 17, size=50)
    herr = np.array([L.ref_hermite_error(F(r), F(nr), F(float(d))) for r, nr, d in zip(rs, nrs, degs)], np.float32)
    # expansion of 6 leaves around a centre and its evaluation
    h = 0.7
    cen = f32([10.3, 7.9])
    leaves = f32(cen + rng.normal(0, 0.4, size=(6, 2)))
    ph = 6
    coef = np.zeros((ph + 1) ** 2, np.float32)
    for lf in leaves:
        L.ref_shift_leaf(P(coef), P(cen), P(f32(lf)), F(1.0), C(ph), F(h))
    qs = f32(cen + rng.normal(0, 1.0, size=(40, 2)))
    ev = np.array([L.ref_evaluate_hermite(P(f32(q)), P(cen), P(coef), C(ph), F(h)) for q in qs], np.float32)
    bits = np.array([L.ref_expand_bits(ctypes.c_uint(v)) for v in range(1024)], np.uint32)
    return dict(ts=ts, herm=herm, rs=rs, nrs=nrs, degs=degs.astype(np.int32), herr=herr, h=np.float32(h), cen=cen,
                leaves=leaves, ph=np.int32(ph), coef=coef, qs=qs, ev=ev, expand_bits=bits)


def gen_karras(L, rng):
    n = 300
    keys = np.sort(rng.integers(0, 1 << 30, size=n).astype(np.uint64))
    keys[50:60] = keys[50]  # duplicate Morton keys
    keys = np.sort(keys)
    k64 = np.ascontiguousarray((keys << np.uint64(32)) | np.arange(n, dtype=np.uint64), np.uint64)
    left = np.zeros(n - 1, np.int32)
    right = np.zeros(n - 1, np.int32)
    parent = np.zeros(2 * n - 1, np.int32)
    L.ref_karras(C(n), P(k64), P(left), P(right), P(parent))
    return dict(keys32=keys.astype(np.uint32), left=left, right=right, parent=parent)


def gen_sampler(L, rng, name, W, H, f, n, K, sd_val, precision, seed):
    pts, nrm = scene_small(rng, n, W, H, f)
    sd = f32(np.full((n, 2), sd_val))
    R = int(np.ceil(np.sqrt(K) - 1e-12))
    uni = f32(rng.uniform(np.finfo(np.float32).tiny, 1.0, size=(W * H * R * K,)))
    uni = np.maximum(uni, np.float32(2.0 ** -24))
    # bandwidth / radius from the oracle (the reference's own reduction is
    # a thrust reduction over device functors); both are then inputs
    import oracle
    h = np.float32(oracle.view_bandwidth(W, H, f, pts, nrm, sd, 0.0))
    radius = np.float32(oracle.cull_radius(h, precision, oracle.LIBM))
    idx = np.zeros((W, H, K), np.int32)
    nvis = np.zeros(1, np.int32)
    keys = np.zeros(n, np.uint32)
    ids = np.zeros(n, np.uint32)
    M = 2 * n - 1
    left, right, degree = np.zeros(M, np.int32), np.zeros(M, np.int32), np.zeros(M, np.int32)
    centre = np.zeros((M, 2), np.float32)
    ov = L.ref_sample_view(C(W), C(H), F(f), C(n), P(pts), F(h), F(radius), C(K), F(precision), P(uni), P(idx),
                           P(nvis), P(keys), P(ids), P(left), P(right), P(degree), P(centre))
    nv = int(nvis[0])
    Mv = max(2 * nv - 1, 0)
    return {f"{name}_{k}": v for k, v in dict(
        W=np.int32(W), H=np.int32(H), f=np.float32(f), K=np.int32(K), precision=np.float32(precision), pts=pts,
        nrm=nrm, sd=sd, uniforms=uni, h=h, radius=radius, indices=idx, n_visible=np.int32(nv), keys=keys[:nv],
        ids=ids[:nv].astype(np.int32), left=left[:Mv], right=right[:Mv], degree=degree[:Mv], centre=centre[:Mv],
        overflows=np.int32(ov)).items()}


def main():
    L = load()
    rng = np.random.default_rng(20221203)
    sets = dict(ewa=gen_ewa(L, rng), pixel_ops=gen_pixel_ops(L, rng), shading=gen_shading(L, rng),
                transform=gen_transform(L, rng), fgt=gen_fgt(L, rng), karras=gen_karras(L, rng))
    smp = {}
    smp.update(gen_sampler(L, rng, "s1", 24, 20, 20.8, 300, 4, 0.01, 0.01, 1))
    smp.update(gen_sampler(L, rng, "s2", 32, 32, 27.7, 900, 8, 0.006, 0.01, 2))
    smp.update(gen_sampler(L, rng, "s3", 20, 16, 17.3, 150, 1, 0.02, 0.001, 3))
    sets["sampler"] = smp
    for k, v in sets.items():
        path = os.path.join(HERE, f"{k}.npz")
        np.savez_compressed(path, **{a: np.asarray(b) for a, b in v.items()})
        print(path, os.path.getsize(path))


if __name__ == "__main__":
    main()
