"""Autotuner for the per-pixel tree descent (the sampler's dominant kernel).

Two choices change the descent's speed but not its result:

* the warp tile: the descent runs one warp per 32-pixel tile, whose width
  along y (``tile_x`` in ``uds_sample_params``: 4, 8, 16 or 32 pixels, the
  height is 32 / tile_x) sets how much of the tree the 32 walks of a warp
  share; every lane walks its own pixel's tree, so the sampled indices are
  identical for every tile shape;
* how the child masses below the expansion frontier are shared out among the
  lanes (``spread``: 0 every lane evaluates its own, 1 spread over the warp);
  the masses are the same calls either way.  Spreading is faster where few
  lanes need masses at a time, evaluating per lane where neighbouring pixels
  descend the same nodes.

``tune_descent`` times the descent of one built view for each (tile_x,
spread) pair with CUDA events and stores the fastest in a JSON cache keyed by
(GPU name, W, H, N, K); ``lookup_config`` is what
``cudaExtensions.sampling.sample`` consults when no ``tile_x`` / ``spread``
is given.  The cache file is ``$UDS_AUTOTUNE_CACHE`` or
``~/.cache/uds_gb300/autotune.json``.

``tune_views`` does the same for a batch of views of different sizes
(``sampling.sample_views``: every view's tree and one descent launch over
all of them), timing the whole call for each configuration, because the best
choice for a batch of small dense views differs from that for its largest
view; its entry is keyed by the list of view sizes.

With ``leaf_sizes`` the sweep also covers the leaf size.  The leaf size does
change the sampled indices (``uds_sample_params.leaf_size``: a round stops at
the first node holding at most max(K, L) splats), so its choice is kept in a
separate cache entry that only ``sampling.sample(leaf_size="auto")`` reads
(``lookup_config(..., leaf=True)``); the default sampling keeps the
reference's rule.
"""
from __future__ import annotations

import itertools
import json
import os
import threading

CANDIDATES = (4, 8, 16, 32)
SPREADS = (0, 1)
LEAF_CANDIDATES = (0, 16, 32)
DEFAULT_TILE = 8

_lock = threading.Lock()
_cache = None


def cache_path() -> str:
    return os.environ.get("UDS_AUTOTUNE_CACHE",
                          os.path.join(os.path.expanduser("~"), ".cache", "uds_gb300", "autotune.json"))


def key(device_name: str, W: int, H: int, N: int, K: int) -> str:
    return f"{device_name}|descent|W={int(W)}|H={int(H)}|N={int(N)}|K={int(K)}"


def views_key(device_name: str, views, N: int, K: int) -> str:
    sizes = ",".join(f"{int(w)}x{int(h)}" for (w, h, _) in views)
    return f"{device_name}|views|{sizes}|N={int(N)}|K={int(K)}"


def _load() -> dict:
    global _cache
    if _cache is None:
        try:
            with open(cache_path()) as f:
                _cache = json.load(f)
        except (OSError, ValueError):
            _cache = {}
    return _cache


def reset() -> None:
    """Forget the in-memory copy (the file is re-read on the next lookup)."""
    global _cache
    with _lock:
        _cache = None


def _entry(k: str, leaf: bool):
    with _lock:
        e = _load().get(k + ("|leaf" if leaf else ""))
    if not e:
        return None
    out = {"tile_x": int(e["tile_x"]), "spread": int(e.get("spread", 0))}
    if leaf:
        out["leaf_size"] = int(e["leaf_size"])
    return out


def lookup_config(device_name: str, W: int, H: int, N: int, K: int, leaf: bool = False):
    """Cached descent configuration for this shape, {"tile_x", "spread"}
    (plus "leaf_size" for the sweep with leaf sizes, ``leaf=True``), or
    None."""
    return _entry(key(device_name, W, H, N, K), leaf)


def lookup_views(device_name: str, views, N: int, K: int, leaf: bool = False):
    """Cached configuration of ``tune_views`` for this list of view sizes, or
    None."""
    return _entry(views_key(device_name, views, N, K), leaf)


def lookup(device_name: str, W: int, H: int, N: int, K: int):
    """Cached tile width for this shape, or None."""
    e = lookup_config(device_name, W, H, N, K)
    return e["tile_x"] if e else None


def lookup_leaf(device_name: str, W: int, H: int, N: int, K: int):
    """Cached (tile_x, leaf_size) of a sweep with leaf sizes, or None."""
    e = lookup_config(device_name, W, H, N, K, leaf=True)
    return (e["tile_x"], e["leaf_size"]) if e else None


def record(device_name: str, W: int, H: int, N: int, K: int, config: dict, timings_ms: dict, views=None) -> None:
    """Store `config` ({"tile_x", "spread"[, "leaf_size"]}) for this shape
    (or for this list of views)."""
    with _lock:
        c = _load()
        entry = {k: int(v) for k, v in config.items()}
        entry["ms"] = {str(k): float(v) for k, v in timings_ms.items()}
        k = key(device_name, W, H, N, K) if views is None else views_key(device_name, views, N, K)
        c[k + ("|leaf" if "leaf_size" in config else "")] = entry
        path = cache_path()
        os.makedirs(os.path.dirname(path), exist_ok=True)
        tmp = path + f".tmp{os.getpid()}"
        with open(tmp, "w") as f:
            json.dump(c, f, indent=1, sort_keys=True)
        os.replace(tmp, path)


def choose(timings_ms: dict):
    """Fastest candidate (ties: the first in sorted order, i.e. the smaller
    tile)."""
    return min(sorted(timings_ms), key=lambda t: timings_ms[t])


def tune_descent(width, height, focallength, points, normals, stdDevs, numSamples, smoothing, precision,
                 view=0, reps=3, candidates=CANDIDATES, timer=None, save=True, leaf_sizes=None, spreads=SPREADS):
    """Time the descent of view `view` for each (tile_x, spread) pair, and
    each leaf size of `leaf_sizes` when given (e.g. LEAF_CANDIDATES), and
    cache the fastest.  `timer(tile_x, spread, leaf_size) -> ms` replaces the
    GPU timing (tests).  Returns (best configuration {"tile_x", "spread"
    [, "leaf_size"]}, {"tile/spread[/leaf]": ms})."""
    import torch
    from ._lib import check, load, stream_ptr
    from .cudaExtensions import sampling
    dev = points.device
    name = torch.cuda.get_device_name(dev) if timer is None else "test-device"
    W, H, N, K = int(width), int(height), int(points.shape[1]), int(numSamples)
    if timer is None:
        tree = sampling.build_tree(width, height, focallength, points[view:view + 1], normals[view:view + 1],
                                   stdDevs[min(view, stdDevs.shape[0] - 1):][:1], K, smoothing, precision)
        prm, ws = tree["_prm"], tree["_ws"]
        L = load()
        idx = torch.empty((W, H, K), dtype=torch.int32, device=dev)
        stream = torch.cuda.current_stream(dev)

        def timer(tx, spread, leaf):
            prm.tile_x = tx
            prm.spread = spread
            prm.leaf_size = leaf
            ts = []
            for r in range(reps + 1):
                e0 = torch.cuda.Event(enable_timing=True)
                e1 = torch.cuda.Event(enable_timing=True)
                e0.record(stream)
                check(L.uds_sample_descent(prm, 0, None, idx.data_ptr(), ws.data_ptr(), ws.numel(),
                                           stream_ptr(dev)), "descent")
                e1.record(stream)
                e1.synchronize()
                if r:
                    ts.append(e0.elapsed_time(e1))
            return min(ts)
    best, timings = _sweep(timer, candidates, spreads, leaf_sizes)
    if save:
        record(name, W, H, N, K, best, timings)
    return best, timings


def _sweep(timer, candidates, spreads, leaf_sizes):
    leaves = tuple(leaf_sizes) if leaf_sizes is not None else (0,)
    pairs = {(int(t), int(s), int(lf)): float(timer(int(t), int(s), int(lf)))
             for t, s, lf in itertools.product(candidates, spreads, leaves)}
    t, s, lf = choose(pairs)
    best = {"tile_x": t, "spread": s}
    if leaf_sizes is not None:
        best["leaf_size"] = lf
        timings = {f"{a}/{b}/{c}": v for (a, b, c), v in pairs.items()}
    else:
        timings = {f"{a}/{b}": v for (a, b, _), v in pairs.items()}
    return best, timings


def tune_views(views, points, normals, stdDevs, numSamples, smoothing, precision, reps=3, candidates=CANDIDATES,
               timer=None, save=True, leaf_sizes=None, spreads=SPREADS):
    """``tune_descent`` for a batch of views of different sizes (``views``: B
    (width, height, focallength); points / normals (B,N,3) in camera space):
    every configuration times a whole ``sampling.sample_views`` call.  The
    result is cached for this list of view sizes, which ``sample_views``
    consults."""
    import torch
    from .cudaExtensions import sampling
    dev = points.device
    name = torch.cuda.get_device_name(dev) if timer is None else "test-device"
    N, K = int(points.shape[1]), int(numSamples)
    if timer is None:
        stream = torch.cuda.current_stream(dev)

        def timer(tx, spread, leaf):
            ts = []
            for r in range(reps + 1):
                e0 = torch.cuda.Event(enable_timing=True)
                e1 = torch.cuda.Event(enable_timing=True)
                e0.record(stream)
                sampling.sample_views(views, points, normals, None, stdDevs, K, smoothing, precision, seed=1,
                                      tile_x=tx, leaf_size=leaf, spread=spread)
                e1.record(stream)
                e1.synchronize()
                if r:
                    ts.append(e0.elapsed_time(e1))
            return min(ts)
    best, timings = _sweep(timer, candidates, spreads, leaf_sizes)
    if save:
        record(name, 0, 0, N, K, best, timings, views=views)
    return best, timings
