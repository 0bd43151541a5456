"""cudaExtensions.sampling (sampling.cpp:48-94, samplingCuda.cu:197-321).

``sample`` builds, per view, the FMM tree over the projected splat centres and
draws ``numSamples`` splat indices per pixel by the sequential-Poisson tree
descent.  Additions over the reference, all optional keyword arguments at the
end so existing calls keep working:

* ``uniforms``: (B,W,H,R,K) float32 in (0,1], R = ceil(sqrt(K)), the random
  numbers consumed by the order sampling (round-major per pixel, candidates in
  Morton order).  Without it Philox4x32-10 uniforms are drawn from ``seed``
  (the reference seeds curand with time(NULL)).
* ``seed``: 64-bit Philox key, or a one-element int64 CUDA tensor holding it
  (read on the device, for CUDA-graph replay); default draws one from
  torch's CPU generator.
* ``h``: (B,) float32 CUDA tensor of bandwidths that replace the computed ones
  (entries <= 0 keep the computed value).
* ``fixed_degree``: 0 (the reference's adaptive expansions) or 4, 6, 8: every
  internal node gets a degree-P expansion built by the M2M shift from its
  children (no reference counterpart; not bit-identical to the oracle).
* ``tile_x``: width of the descent's 32-pixel warp tiles (4, 8, 16, 32);
  default: the autotuner's cached choice for this shape (see ``autotune``),
  else 8.  The indices do not depend on it.
* ``spread``: 0 or 1, how the descent shares out the child masses below the
  expansion frontier among a warp's lanes (K <= 8); default: the
  autotuner's cached choice, else 0.  The indices do not depend on it.
* ``leaf_size``: 0 or <= K (default): the reference's single-splat leaves.
  K < L <= 64 (no reference counterpart): leaf buckets of L splats; each round
  of the descent stops at the first node holding <= L splats and
  order-samples over all of them with their exact Gaussians, so fewer
  levels are descended below the expansion frontier.  The indices differ
  from the default's (the oracle has the same rule); ``uniforms`` is then
  (B,W,H,R,L).  ``"auto"``: the (tile, leaf size) pair the autotuner's
  tile x leaf sweep cached for this shape (``autotune.lookup_leaf``), else
  the default rule.
* ``return_stats``: also return the per-view record (h, cull radius, visible
  splats, stored coefficients, demoted nodes, trace overflows) as a (B,8)
  tensor viewed from uds_view_stats.

``sample_stochastic`` is a second sampling mode with no reference
counterpart: K independent mass-proportional descents per pixel, returning the
indices and each draw's path probability q (for importance-weighted
estimators).
"""
from __future__ import annotations

import math

import torch

from .._lib import SampleParams, ViewDesc, Workspace, check, load, need, ptr, stream_ptr

MAX_DEGREE = 16


def num_rounds(K: int) -> int:
    return int(math.ceil(math.sqrt(K) - 1e-12))


def params(width, height, focallength, points, stdDevs, numSamples, smoothing, precision, seed=0,
           max_degree=MAX_DEGREE, coef_pool=0, tile_x=0, fixed_degree=0, leaf_size=0, spread=0) -> SampleParams:
    """``seed``: an int, or a one-element int64 CUDA tensor whose value the
    kernels read when they run (a captured CUDA graph then draws new numbers
    after the tensor is updated)."""
    prm = SampleParams(B=points.shape[0], N=points.shape[1], W=int(width), H=int(height), K=int(numSamples),
                       focal=float(focallength), smoothing=float(smoothing), precision=float(precision),
                       max_degree=int(max_degree), std_batch=stdDevs.shape[0], coef_pool=int(coef_pool or 0),
                       seed=0, seed_dev=None, tile_x=int(tile_x or 0), fixed_degree=int(fixed_degree or 0),
                       leaf_size=int(leaf_size or 0), spread=int(spread or 0))
    if isinstance(seed, torch.Tensor):
        if seed.dtype != torch.int64 or seed.numel() != 1 or seed.device != points.device:
            raise ValueError("a seed tensor must be one int64 element on the points' device")
        prm.seed_dev = seed.data_ptr()
    else:
        prm.seed = int(seed) & 0xFFFFFFFFFFFFFFFF
    return prm


def workspace_bytes(prm: SampleParams) -> int:
    n = load().uds_sample_workspace_size(prm)
    if n == 0:
        raise ValueError("invalid sampling parameters")
    return n


def _check(points, normals, stdDevs):
    need(points, "points")
    need(normals, "normals", device=points.device)
    need(stdDevs, "stdDevs", device=points.device)
    if points.dim() != 3 or points.shape[2] != 3 or normals.shape != points.shape:
        raise ValueError("points and normals must be (B,N,3)")
    if stdDevs.dim() != 3 or stdDevs.shape[2] != 2 or stdDevs.shape[1] != points.shape[1] or \
            stdDevs.shape[0] not in (1, points.shape[0]):
        raise ValueError("stdDevs must be (1|B,N,2)")


def _descent(points, width, height, numSamples, tile_x=None, leaf_size=0, spread=None):
    """(tile_x, leaf_size, spread) of the descent: the given values, else the
    autotuner's cached choices for this shape (``leaf_size="auto"``: those of
    its sweep with leaf sizes), else the defaults (8, 0, 0)."""
    from .. import autotune
    auto_leaf = leaf_size == "auto"
    if tile_x and spread is not None and not auto_leaf:
        return int(tile_x), int(leaf_size or 0), int(spread)
    name = _device_name(points.device)
    e = autotune.lookup_config(name, width, height, points.shape[1], numSamples, leaf=auto_leaf)
    if e is None and auto_leaf:
        e = autotune.lookup_config(name, width, height, points.shape[1], numSamples)
    e = e or {}
    return (int(tile_x) if tile_x else e.get("tile_x", autotune.DEFAULT_TILE),
            e.get("leaf_size", 0) if auto_leaf else int(leaf_size or 0),
            int(spread) if spread is not None else e.get("spread", 0))


def _descent_views(views, points, numSamples, tile_x=None, leaf_size=0, spread=None):
    """``_descent`` for a batch of views: the cached choices of
    ``autotune.tune_views`` for this list of view sizes, else those for the
    first view's shape."""
    from .. import autotune
    auto_leaf = leaf_size == "auto"
    if not (tile_x and spread is not None and not auto_leaf):
        e = autotune.lookup_views(_device_name(points.device), views, points.shape[1], numSamples, leaf=auto_leaf)
        if e is not None:
            return (int(tile_x) if tile_x else e["tile_x"], e.get("leaf_size", 0) if auto_leaf else int(leaf_size or 0),
                    int(spread) if spread is not None else e["spread"])
    W0, H0, _ = views[0]
    return _descent(points, W0, H0, numSamples, tile_x, leaf_size, spread)


_device_names = {}


def _device_name(dev):
    name = _device_names.get(dev.index)
    if name is None:
        name = _device_names[dev.index] = torch.cuda.get_device_name(dev)
    return name


def sample(width: int, height: int, focallength: float, points, normals, colors, stdDevs, numSamples: int,
           smoothing: float, precision: float, uniforms=None, seed=None, h=None, return_stats=False,
           max_degree=MAX_DEGREE, coef_pool=0, tile_x=None, fixed_degree=0, leaf_size=0, spread=None):
    _check(points, normals, stdDevs)
    dev = points.device
    B = points.shape[0]
    K = int(numSamples)
    if seed is None:
        seed = int(torch.randint(0, 2 ** 62, (1,)).item())
    tile_x, leaf_size, spread = _descent(points, width, height, K, tile_x, leaf_size, spread)
    prm = params(width, height, focallength, points, stdDevs, K, smoothing, precision, seed, max_degree, coef_pool,
                 tile_x, fixed_degree, leaf_size, spread)
    if uniforms is not None:
        need(uniforms, "uniforms", device=dev)
        R, M = num_rounds(K), max(K, int(leaf_size or 0))
        if tuple(uniforms.shape) != (B, int(width), int(height), R, M):
            raise ValueError(f"uniforms must be (B,W,H,{R},{M})")
    if h is not None:
        need(h, "h", device=dev)
        if h.numel() != B:
            raise ValueError("h must have B entries")
    L = load()
    ws = Workspace.get(dev, workspace_bytes(prm), "sample")
    indices = torch.empty((B, int(width), int(height), K), dtype=torch.int32, device=dev)
    stats = torch.empty((B, 8), dtype=torch.float32, device=dev) if return_stats else None
    check(L.uds_sample(prm, ptr(points), ptr(normals), ptr(stdDevs), ptr(uniforms), ptr(h), ptr(indices), ptr(stats),
                       ptr(ws), ws.numel(), stream_ptr(dev)), "sampling sample")
    if return_stats:
        return indices, view_stats(stats)
    return indices


def sample_views(views, points, normals, colors, stdDevs, numSamples: int, smoothing: float, precision: float,
                 seed=None, h=None, return_stats=False, max_degree=MAX_DEGREE, coef_pool=0, tile_x=None,
                 fixed_degree=0, leaf_size=0, spread=None):
    """sampling.sample for B views of different sizes in one call (no
    reference counterpart): ``views`` is a list of B (width, height,
    focallength); points / normals (B,N,3), stdDevs (1|B,N,2).  Every view's
    tree is built, then one descent launch covers all views' pixels (K <= 8).
    Returns the list of (1, W_b, H_b, K) int32 index tensors (views of one
    packed buffer), and the per-view stats when asked.  View b draws the
    Philox uniforms of view b of ``sample`` on a view of that size."""
    _check(points, normals, stdDevs)
    dev = points.device
    B, K = points.shape[0], int(numSamples)
    if len(views) != B:
        raise ValueError("one (width, height, focallength) per view of points")
    if seed is None:
        seed = int(torch.randint(0, 2 ** 62, (1,)).item())
    W0, H0, f0 = views[0]
    tile_x, leaf_size, spread = _descent_views(views, points, K, tile_x, leaf_size, spread)
    prm = params(W0, H0, f0, points, stdDevs, K, smoothing, precision, seed, max_degree, coef_pool, tile_x,
                 fixed_degree, leaf_size, spread)
    desc = (ViewDesc * B)(*[ViewDesc(int(w), int(hh), float(f), 0) for (w, hh, f) in views])
    if h is not None:
        need(h, "h", device=dev)
        if h.numel() != B:
            raise ValueError("h must have B entries")
    L = load()
    ws = Workspace.get(dev, workspace_bytes(prm), "sample")
    sizes = [int(w) * int(hh) * K for (w, hh, _) in views]
    packed = torch.empty(sum(sizes), dtype=torch.int32, device=dev)
    stats = torch.empty((B, 8), dtype=torch.float32, device=dev) if return_stats else None
    check(L.uds_sample_views(prm, desc, ptr(points), ptr(normals), ptr(stdDevs), ptr(h), ptr(packed), ptr(stats),
                             ptr(ws), ws.numel(), stream_ptr(dev)), "sampling sample_views")
    out, o = [], 0
    for (w, hh, _), n in zip(views, sizes):
        out.append(packed[o:o + n].view(1, int(w), int(hh), K))
        o += n
    if return_stats:
        return out, view_stats(stats)
    return out


def sample_stochastic(width: int, height: int, focallength: float, points, normals, stdDevs, numSamples: int,
                      smoothing: float, precision: float, seed=None, h=None, return_stats=False,
                      max_degree=MAX_DEGREE, coef_pool=0):
    """K independent draws per pixel, each descending the FGT tree with
    child-mass-proportional probabilities.  Returns (indices (B,W,H,K) int32,
    probs (B,W,H,K) float32 path probabilities; -1 / 0 where no draw)."""
    _check(points, normals, stdDevs)
    dev = points.device
    B = points.shape[0]
    K = int(numSamples)
    if seed is None:
        seed = int(torch.randint(0, 2 ** 62, (1,)).item())
    prm = params(width, height, focallength, points, stdDevs, K, smoothing, precision, seed, max_degree, coef_pool)
    if h is not None:
        need(h, "h", device=dev)
        if h.numel() != B:
            raise ValueError("h must have B entries")
    L = load()
    ws = Workspace.get(dev, workspace_bytes(prm), "sample")
    indices = torch.empty((B, int(width), int(height), K), dtype=torch.int32, device=dev)
    probs = torch.empty((B, int(width), int(height), K), dtype=torch.float32, device=dev)
    stats = torch.empty((B, 8), dtype=torch.float32, device=dev) if return_stats else None
    check(L.uds_sample_stochastic(prm, ptr(points), ptr(normals), ptr(stdDevs), ptr(h), ptr(indices), ptr(probs),
                                  ptr(stats), ptr(ws), ws.numel(), stream_ptr(dev)), "sampling sample_stochastic")
    if return_stats:
        return indices, probs, view_stats(stats)
    return indices, probs


def view_stats(stats: torch.Tensor) -> dict:
    """Decode a (B,8) uds_view_stats tensor (synchronises)."""
    s = stats.detach().cpu()
    ints = s.view(torch.int32)
    return dict(h=s[:, 0].clone(), radius=s[:, 1].clone(), n_visible=ints[:, 2].clone(), n_coefs=ints[:, 3].clone(),
                demoted=ints[:, 4].clone(), overflow=ints[:, 5].clone())


def build_tree(width, height, focallength, points, normals, stdDevs, numSamples, smoothing, precision, view=0,
               h=None, max_degree=MAX_DEGREE, coef_pool=0, fixed_degree=0):
    """Build one view's tree and return its arrays (test / debug helper of
    uds_tree_build).  Keeps the workspace for fgt_eval."""
    _check(points, normals, stdDevs)
    dev = points.device
    N = points.shape[1]
    prm = params(width, height, focallength, points, stdDevs, numSamples, smoothing, precision, 0, max_degree,
                 coef_pool, 0, fixed_degree)
    L = load()
    ws = Workspace.get(dev, workspace_bytes(prm), "tree")
    M = max(2 * N - 1, 1)
    out = dict(keys=torch.empty(max(N, 1), dtype=torch.int32, device=dev),
               ids=torch.empty(max(N, 1), dtype=torch.int32, device=dev),
               left=torch.empty(M, dtype=torch.int32, device=dev), right=torch.empty(M, dtype=torch.int32, device=dev),
               parent=torch.empty(M, dtype=torch.int32, device=dev), count=torch.empty(M, dtype=torch.int32, device=dev),
               degree=torch.empty(M, dtype=torch.int32, device=dev),
               centre=torch.empty((M, 2), dtype=torch.float32, device=dev),
               box=torch.empty((M, 4), dtype=torch.float32, device=dev))
    stats = torch.empty((1, 8), dtype=torch.float32, device=dev)
    if h is not None:
        need(h, "h", device=dev)
    check(L.uds_tree_build(prm, int(view), ptr(points), ptr(normals), ptr(stdDevs), ptr(h), ptr(stats),
                           ptr(out["keys"]), ptr(out["ids"]), ptr(out["left"]), ptr(out["right"]), ptr(out["parent"]),
                           ptr(out["count"]), ptr(out["degree"]), ptr(out["centre"]), ptr(out["box"]), ptr(ws),
                           ws.numel(), stream_ptr(dev)), "tree build")
    st = view_stats(stats)
    n = int(st["n_visible"][0])
    Mn = max(2 * n - 1, 0)
    res = {k: (v[:n] if k in ("keys", "ids") else v[:Mn]).cpu() for k, v in out.items()}
    res.update({k: float(v[0]) if k in ("h", "radius") else int(v[0]) for k, v in st.items()})
    res["_prm"] = prm
    res["_ws"] = ws
    return res


def fgt_eval(tree: dict, nodes, queries):
    """getWeight of (node, query) pairs on the tree last built by build_tree."""
    ws = tree["_ws"]
    nodes = need(nodes, "nodes", torch.int32)
    queries = need(queries, "queries", device=nodes.device)
    out = torch.empty(nodes.numel(), dtype=torch.float32, device=nodes.device)
    check(load().uds_fgt_eval(tree["_prm"], nodes.numel(), ptr(nodes), ptr(queries), ptr(out), ptr(ws), ws.numel(),
                              stream_ptr(nodes.device)), "fgt eval")
    return out
