"""Python bindings of the CPU oracle (oracle/uds_oracle.c).

TEST INFRASTRUCTURE ONLY.  Only tests/, ``__graft_entry__.smoke()`` and the CPU
legs of ``bench.py`` import this package, to check or to time the CUDA path;
the product package never does.

All functions take and return numpy arrays in the reference's layouts
(splats ``(1|B, N, c)``, pixels ``(B, W, H, ...)``).  The library is built on
first use with ``make -C oracle oracle`` when it is missing.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
import threading

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liboracle.so")
REF_PATH = os.path.join(HERE, "_ref", "libudsref.so")

DET = 0   # arithmetic the CUDA path reproduces bit for bit
LIBM = 1  # the reference's own arithmetic (libm exp/log/pow)

_lock = threading.Lock()
_lib = None

_f32p = ctypes.POINTER(ctypes.c_float)
_f64p = ctypes.POINTER(ctypes.c_double)
_i32p = ctypes.POINTER(ctypes.c_int)
_u32p = ctypes.POINTER(ctypes.c_uint)


def build(force: bool = False) -> str:
    """Compile liboracle.so with the committed Makefile."""
    if force or not os.path.exists(LIB_PATH):
        subprocess.run(["make", "-s", "-C", HERE, "oracle"], check=True)
    return LIB_PATH


def lib():
    global _lib
    with _lock:
        if _lib is None:
            build()
            L = ctypes.CDLL(LIB_PATH)
            L.orc_det_expf.restype = ctypes.c_float
            L.orc_det_expf.argtypes = [ctypes.c_float]
            L.orc_det_logf.restype = ctypes.c_float
            L.orc_det_logf.argtypes = [ctypes.c_float]
            L.orc_view_bandwidth.restype = ctypes.c_float
            L.orc_cull_radius.restype = ctypes.c_float
            L.orc_cull_radius.argtypes = [ctypes.c_float, ctypes.c_float, ctypes.c_int]
            L.orc_ewa_weight.restype = ctypes.c_float
            L.orc_tree_build.restype = ctypes.c_void_p
            L.orc_tree_free.argtypes = [ctypes.c_void_p]
            L.orc_tree_size.restype = ctypes.c_int
            L.orc_tree_size.argtypes = [ctypes.c_void_p]
            L.orc_tree_num_coefs.restype = ctypes.c_long
            L.orc_tree_num_coefs.argtypes = [ctypes.c_void_p]
            L.orc_tree_node_weight.restype = ctypes.c_float
            L.orc_tree_node_weight.argtypes = [ctypes.c_void_p, ctypes.c_int, _f32p, ctypes.c_int]
            L.orc_tree_direct_weight.restype = ctypes.c_double
            L.orc_tree_direct_weight.argtypes = [ctypes.c_void_p, ctypes.c_int, _f64p]
            L.orc_num_rounds.restype = ctypes.c_int
            L.orc_num_threads.restype = ctypes.c_int
            _lib = L
    return _lib


def _f(a):
    return np.ascontiguousarray(a, dtype=np.float32)


def _i(a):
    return np.ascontiguousarray(a, dtype=np.int32)


def P(a):
    if a is None:
        return None
    if a.dtype == np.float32:
        return a.ctypes.data_as(_f32p)
    if a.dtype == np.float64:
        return a.ctypes.data_as(_f64p)
    if a.dtype == np.int32:
        return a.ctypes.data_as(_i32p)
    if a.dtype == np.uint32:
        return a.ctypes.data_as(_u32p)
    raise TypeError(a.dtype)


C = ctypes.c_int
F = ctypes.c_float


def det_expf(x: float) -> float:
    return lib().orc_det_expf(float(x))


def det_logf(x: float) -> float:
    return lib().orc_det_logf(float(x))


def num_rounds(K: int) -> int:
    return lib().orc_num_rounds(int(K))


def num_threads() -> int:
    return lib().orc_num_threads()


def philox_uniforms(seed: int, view: int, pixel: int, rnd: int, K: int) -> np.ndarray:
    out = np.zeros(K, np.float32)
    lib().orc_philox_uniforms(ctypes.c_uint64(seed), ctypes.c_uint32(view), ctypes.c_uint32(pixel),
                              ctypes.c_uint32(rnd), C(K), P(out))
    return out


# ---------------------------------------------------------------- transform
def transform_forward(M, v, affine=True):
    M, v = _f(M), _f(v)
    B, N = M.shape[0], v.shape[1]
    out = np.zeros((B, N, 3), np.float32)
    lib().orc_transform_forward(C(int(affine)), C(B), P(M), C(v.shape[0]), C(N), P(v), P(out))
    return out


def transform_backward(g, M, v, affine=True):
    g, M, v = _f(g), _f(M), _f(v)
    B, N = M.shape[0], v.shape[1]
    gM = np.zeros_like(M)
    gv = np.zeros_like(v)
    lib().orc_transform_backward(C(int(affine)), C(B), P(g), P(M), C(v.shape[0]), C(N), P(v), P(gM), P(gv))
    return gM, gv


# ---------------------------------------------------------------------- EWA
def to_screenspace(W, H, f, pts):
    pts = _f(pts).reshape(-1, 3)
    out = np.zeros((pts.shape[0], 2), np.float32)
    lib().orc_to_screenspace(C(pts.shape[0]), F(W), F(H), F(f), P(pts), P(out))
    return out


def splat_forward(W, H, f, idx, pts, nrm, sd, smoothing):
    idx, pts, nrm, sd = _i(idx), _f(pts), _f(nrm), _f(sd)
    B, _, _, K = idx.shape
    w = np.zeros(idx.shape, np.float32)
    lib().orc_splat_forward(C(B), C(W), C(H), C(K), F(f), P(idx), P(pts), P(nrm), P(sd), C(sd.shape[0]),
                            C(pts.shape[1]), F(smoothing), P(w))
    return w


def splat_backward(W, H, f, gin, idx, pts, nrm, sd, smoothing):
    gin, idx, pts, nrm, sd = _f(gin), _i(idx), _f(pts), _f(nrm), _f(sd)
    B, _, _, K = idx.shape
    gp, gn, gs = np.zeros_like(pts), np.zeros_like(nrm), np.zeros_like(sd)
    lib().orc_splat_backward(C(B), C(W), C(H), C(K), F(f), P(gin), P(idx), P(pts), P(nrm), P(sd),
                             C(sd.shape[0]), C(pts.shape[1]), F(smoothing), P(gp), P(gn), P(gs))
    return gp, gn, gs


def ewa_grad(pixel, W, H, f, p, n, sd, smoothing):
    """FP64 gradient of the (unclamped) EWA weight of one (pixel, splat) pair."""
    gp = np.zeros(3, np.float64)
    gn = np.zeros(3, np.float64)
    gs = np.zeros(2, np.float64)
    lib().orc_ewa_grad(P(_f(pixel)), F(W), F(H), F(f), P(_f(p)), P(_f(n)), P(_f(sd)), F(smoothing),
                       P(gp), P(gn), P(gs))
    return gp, gn, gs


# ------------------------------------------------------------- compositing
def filter_forward(idx, w, W, H, f, pts, nrm, return_order=False):
    idx, w, pts, nrm = _i(idx), _f(w), _f(pts), _f(nrm)
    B, _, _, K = idx.shape
    out = np.zeros_like(w)
    order = np.zeros(idx.shape, np.int32) if return_order else None
    lib().orc_filter_forward(C(B), C(W), C(H), C(K), P(idx), P(w), F(f), C(pts.shape[0]), C(pts.shape[1]),
                             P(pts), P(nrm), P(out), P(order))
    return (out, order) if return_order else out


def filter_backward(idx, w, gin, W, H, f, pts, nrm):
    idx, w, gin, pts, nrm = _i(idx), _f(w), _f(gin), _f(pts), _f(nrm)
    B, _, _, K = idx.shape
    out = np.zeros_like(w)
    lib().orc_filter_backward(C(B), C(W), C(H), C(K), P(idx), P(w), P(gin), F(f), C(pts.shape[0]),
                              C(pts.shape[1]), P(pts), P(nrm), P(out))
    return out


# ------------------------------------------------------------ interpolation
def interp_forward(idx, w, attr):
    idx, w, attr = _i(idx), _f(w), _f(attr)
    B, W, H, K = idx.shape
    Cn = attr.shape[2]
    out = np.zeros((B, W, H, Cn), np.float32)
    lib().orc_interp_forward(C(B), C(W), C(H), C(K), P(idx), P(w), C(attr.shape[0]), C(attr.shape[1]), C(Cn),
                             P(attr), P(out))
    return out


def chain64_forward(W, H, f, idx, pts, nrm, sd, smoothing, attr):
    """EWA -> compositing -> interpolation of one view in FP64 for fixed
    indices (W,H,K); pts/nrm (N,3), sd (N,2), attr (N,C) -> image (W,H,C)
    float64."""
    idx = _i(idx)
    d = lambda a: np.ascontiguousarray(a, dtype=np.float64)  # noqa: E731
    pts, nrm, sd, attr = d(pts), d(nrm), d(sd), d(attr)
    K = idx.shape[-1]
    Cn = attr.shape[1]
    img = np.zeros((W, H, Cn), np.float64)
    lib().orc_chain64_forward(C(W), C(H), C(K), ctypes.c_double(f), P(idx), C(pts.shape[0]), P(pts), P(nrm), P(sd),
                              ctypes.c_double(smoothing), C(Cn), P(attr), P(img))
    return img


def interp_backward(gin, idx, w, attr):
    gin, idx, w, attr = _f(gin), _i(idx), _f(w), _f(attr)
    B, W, H, K = idx.shape
    Cn = attr.shape[2]
    gw = np.zeros_like(w)
    ga = np.zeros_like(attr)
    lib().orc_interp_backward(C(B), C(W), C(H), C(K), P(gin), P(idx), P(w), C(attr.shape[0]), C(attr.shape[1]),
                              C(Cn), P(attr), P(gw), P(ga))
    return gw, ga


# --------------------------------------------------------------- pixelgather
def pixel_scatter(idx, values):
    idx, values = _i(idx), _f(values)
    B, W, H, K = idx.shape
    N, Cn = values.shape[1], values.shape[2]
    out = np.zeros((B, W, H, K, Cn), np.float32)
    lib().orc_pixel_scatter(C(B), C(W), C(H), C(K), P(idx), C(N), C(Cn), P(values), P(out))
    return out


def pixel_gather(idx, values, N):
    idx, values = _i(idx), _f(values)
    B, W, H, K = idx.shape
    Cn = values.shape[4]
    out = np.zeros((B, N, Cn), np.float32)
    lib().orc_pixel_gather(C(B), C(W), C(H), C(K), P(idx), C(N), C(Cn), P(values), P(out))
    return out


def nearest_samples(idx, w, pts, M):
    idx, w, pts = _i(idx), _f(w), _f(pts).reshape(-1, 3)
    B, W, H, K = idx.shape
    N = pts.shape[0]
    out = np.full((N, M), -1, np.int32)
    lib().orc_nearest_samples(C(B), C(W), C(H), C(K), P(idx), P(w), C(N), P(pts), C(M), P(out))
    return out


# ------------------------------------------------------------------ shading
def shade_forward(dirs, I, nrm, dif):
    dirs, I, nrm, dif = _f(dirs), _f(I), _f(nrm), _f(dif)
    B = nrm.shape[0]
    Pn = int(np.prod(nrm.shape[1:-1]))
    out = np.zeros_like(nrm)
    lib().orc_shade_forward(C(B), C(Pn), C(I.shape[1]), P(dirs), P(I), C(I.shape[0]), P(nrm), P(dif), P(out))
    return out


def shade_backward(gin, dirs, I, nrm, dif):
    gin, dirs, I, nrm, dif = _f(gin), _f(dirs), _f(I), _f(nrm), _f(dif)
    B = nrm.shape[0]
    Pn = int(np.prod(nrm.shape[1:-1]))
    gd, gI, gn, gdf = np.zeros_like(dirs), np.zeros_like(I), np.zeros_like(nrm), np.zeros_like(dif)
    lib().orc_shade_backward(C(B), C(Pn), C(I.shape[1]), P(gin), P(dirs), P(I), C(I.shape[0]), P(nrm), P(dif),
                             P(gd), P(gI), P(gn), P(gdf))
    return gd, gI, gn, gdf


def shade_sh_forward(coef, nrm, dif):
    coef, nrm, dif = _f(coef), _f(nrm), _f(dif)
    B = nrm.shape[0]
    Pn = int(np.prod(nrm.shape[1:-1]))
    out = np.zeros_like(nrm)
    lib().orc_shade_sh_forward(C(B), C(Pn), P(coef), C(coef.shape[0]), P(nrm), P(dif), P(out))
    return out


def shade_sh_backward(gin, coef, nrm, dif):
    gin, coef, nrm, dif = _f(gin), _f(coef), _f(nrm), _f(dif)
    B = nrm.shape[0]
    Pn = int(np.prod(nrm.shape[1:-1]))
    gc, gn, gd = np.zeros_like(coef), np.zeros_like(nrm), np.zeros_like(dif)
    lib().orc_shade_sh_backward(C(B), C(Pn), P(gin), P(coef), C(coef.shape[0]), P(nrm), P(dif), P(gc), P(gn), P(gd))
    return gc, gn, gd


# ------------------------------------------------------------------ sampler
def view_bandwidth(W, H, f, pts, nrm, sd, smoothing):
    pts, nrm, sd = _f(pts).reshape(-1, 3), _f(nrm).reshape(-1, 3), _f(sd).reshape(-1, 2)
    return lib().orc_view_bandwidth(C(W), C(H), F(f), C(pts.shape[0]), P(pts), P(nrm), P(sd), F(smoothing))


def cull_radius(h, precision, flavour=DET):
    return lib().orc_cull_radius(F(h), F(precision), C(flavour))


class Tree:
    """One view's FMM tree as the oracle builds it."""

    def __init__(self, W, H, f, pts, h, radius, precision, max_degree=16, coef_pool=-1, flavour=DET):
        self.pts = _f(pts).reshape(-1, 3)
        self.flavour = flavour
        self.h = float(h)
        self.ptr = lib().orc_tree_build(C(W), C(H), F(f), C(self.pts.shape[0]), P(self.pts), F(h), F(radius),
                                        F(precision), C(max_degree), ctypes.c_long(coef_pool), C(flavour))
        if not self.ptr:
            raise MemoryError("oracle tree build failed")
        self.n = lib().orc_tree_size(self.ptr)
        self.num_coefs = lib().orc_tree_num_coefs(self.ptr)

    def __del__(self):
        if getattr(self, "ptr", None):
            lib().orc_tree_free(self.ptr)
            self.ptr = None

    def export(self):
        n = self.n
        M = max(2 * n - 1, 0)
        d = dict(keys=np.zeros(n, np.uint32), ids=np.zeros(n, np.int32), left=np.zeros(M, np.int32),
                 right=np.zeros(M, np.int32), parent=np.zeros(M, np.int32), count=np.zeros(M, np.int32),
                 degree=np.zeros(M, np.int32), centre=np.zeros((M, 2), np.float32),
                 box=np.zeros((M, 4), np.float32), leafxy=np.zeros((n, 2), np.float32))
        lib().orc_tree_export(ctypes.c_void_p(self.ptr), P(d["keys"]), P(d["ids"]), P(d["left"]), P(d["right"]),
                              P(d["parent"]), P(d["count"]), P(d["degree"]), P(d["centre"]), P(d["box"]),
                              P(d["leafxy"]))
        return d

    def node_weight(self, node, query, flavour=None):
        q = np.asarray(query, np.float32)
        fl = self.flavour if flavour is None else flavour
        return lib().orc_tree_node_weight(ctypes.c_void_p(self.ptr), C(node), P(q), C(fl))

    def direct_weight(self, node, query):
        q = np.asarray(query, np.float64)
        return lib().orc_tree_direct_weight(ctypes.c_void_p(self.ptr), C(node), P(q))

    def sample_stochastic(self, W, H, K, precision, seed=0, view=0, x0=0, x1=None, flavour=None):
        """Stochastic mode: (indices (W,H,K), path probabilities (W,H,K))."""
        idx = np.full((W, H, K), -1, np.int32)
        prob = np.zeros((W, H, K), np.float32)
        fl = self.flavour if flavour is None else flavour
        st = lib().orc_tree_sample_stochastic(ctypes.c_void_p(self.ptr), C(W), C(H), C(K), F(precision),
                                              ctypes.c_uint64(seed), ctypes.c_uint32(view), C(x0),
                                              C(W if x1 is None else x1), C(fl), P(idx), P(prob))
        if st != 0:
            raise RuntimeError("oracle stochastic sampler: path deeper than 64 levels")
        return idx, prob

    def candidates(self, K, precision, i, j, flavour=None):
        """(splat ids, leaf masses) of every candidate entry of pixel (i, j)."""
        R = num_rounds(K)
        ids = np.zeros(R * K, np.int32)
        p = np.zeros(R * K, np.float32)
        fl = self.flavour if flavour is None else flavour
        m = lib().orc_tree_candidates(ctypes.c_void_p(self.ptr), C(K), F(precision), C(i), C(j), C(fl), P(ids), P(p))
        if m < 0:
            raise RuntimeError("oracle sampler trace overflow")
        return ids[:m], p[:m]

    def sample(self, W, H, K, precision, uniforms=None, seed=0, view=0, x0=0, x1=None, flavour=None, leaf_size=0):
        """Poisson descent: indices (W,H,K).  ``leaf_size`` > K: rounds stop at
        the first node holding <= leaf_size splats (uniforms then
        (W,H,R,max(K,leaf_size)))."""
        idx = np.full((W, H, K), -1, np.int32)
        u = None if uniforms is None else _f(uniforms)
        fl = self.flavour if flavour is None else flavour
        st = lib().orc_tree_sample_leaf(ctypes.c_void_p(self.ptr), C(W), C(H), C(K), C(leaf_size), F(precision), P(u),
                                        ctypes.c_uint64(seed), ctypes.c_uint32(view), C(x0),
                                        C(W if x1 is None else x1), C(fl), P(idx))
        if st != 0:
            raise RuntimeError("oracle sampler trace overflow" if st == -1 else "oracle sampler: leaf size > 64")
        return idx


def sample_fp64(tree, W, H, K, precision, seed=0, view=0, x0=0, x1=None, leaf_size=0):
    """The estimator evaluated directly in FP64 on an oracle Tree (direct Gauss
    sums instead of Hermite expansions; same descent and order sampling with
    Philox uniforms): indices (W,H,K)."""
    idx = np.full((W, H, K), -1, np.int32)
    st = lib().orc_tree_sample_fp64_leaf(ctypes.c_void_p(tree.ptr), C(W), C(H), C(K), C(leaf_size),
                                         ctypes.c_double(precision), ctypes.c_uint64(seed), ctypes.c_uint32(view),
                                         C(x0), C(W if x1 is None else x1), P(idx))
    if st != 0:
        raise RuntimeError("oracle FP64 sampler: path deeper than 64 levels")
    return idx


def sample_view_stochastic(W, H, f, pts, nrm, sd, K, smoothing, precision, h=0.0, seed=0, view=0, flavour=DET):
    """Stochastic sampling mode for one view: (indices (W,H,K), probs (W,H,K))."""
    pts, nrm, sd = _f(pts).reshape(-1, 3), _f(nrm).reshape(-1, 3), _f(sd).reshape(-1, 2)
    hh = h if h > 0 else view_bandwidth(W, H, f, pts, nrm, sd, smoothing)
    t = Tree(W, H, f, pts, hh, cull_radius(hh, precision, flavour), precision, flavour=flavour)
    return t.sample_stochastic(W, H, K, precision, seed=seed, view=view)


def sample_view(W, H, f, pts, nrm, sd, K, smoothing, precision, h=0.0, uniforms=None, seed=0, view=0,
                flavour=DET):
    """sampling.sample for one view.  Returns (indices (W,H,K) int32, stats)."""
    pts, nrm, sd = _f(pts).reshape(-1, 3), _f(nrm).reshape(-1, 3), _f(sd).reshape(-1, 2)
    idx = np.full((W, H, K), -1, np.int32)
    stats = np.zeros(4, np.float32)
    u = None if uniforms is None else _f(uniforms)
    st = lib().orc_sample_view(C(W), C(H), F(f), C(pts.shape[0]), P(pts), P(nrm), P(sd), C(K), F(smoothing),
                               F(precision), F(h), P(u), ctypes.c_uint64(seed), ctypes.c_uint32(view), C(flavour),
                               P(idx), P(stats))
    if st != 0:
        raise RuntimeError(f"oracle sampler failed ({st})")
    return idx, dict(h=float(stats[0]), radius=float(stats[1]), n_visible=int(stats[2]), n_coefs=int(stats[3]))
