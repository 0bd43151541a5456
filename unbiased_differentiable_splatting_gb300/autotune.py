"""Autotuner for the per-pixel tree descent (the sampler's dominant kernel).

The descent runs one warp per 32-pixel tile; the tile's width along y
(``tile_x`` in ``uds_sample_params``: 4, 8, 16 or 32 pixels, the height is
32 / tile_x) sets how much of the tree the 32 walks of a warp share, and so
the speed, but not the result: every lane walks its own pixel's tree, so the
sampled indices are identical for every tile shape.

``tune_descent`` times the descent of one built view for each candidate with
CUDA events and stores the fastest in a JSON cache keyed by (GPU name, W, H,
N, K); ``lookup`` is what ``cudaExtensions.sampling.sample`` consults when no
``tile_x`` is given.  The cache file is ``$UDS_AUTOTUNE_CACHE`` or
``~/.cache/uds_gb300/autotune.json``.

With ``leaf_sizes`` the sweep covers tile x leaf size.  The leaf size does
change the sampled indices (``uds_sample_params.leaf_size``: a round stops at
the first node holding at most max(K, L) splats), so its choice is kept in a
separate cache entry that only ``sampling.sample(leaf_size="auto")`` reads
(``lookup_leaf``); the default sampling keeps the reference's rule.
"""
from __future__ import annotations

import json
import os
import threading

CANDIDATES = (4, 8, 16, 32)
LEAF_CANDIDATES = (0, 16, 32)
DEFAULT_TILE = 8

_lock = threading.Lock()
_cache = None


def cache_path() -> str:
    return os.environ.get("UDS_AUTOTUNE_CACHE",
                          os.path.join(os.path.expanduser("~"), ".cache", "uds_gb300", "autotune.json"))


def key(device_name: str, W: int, H: int, N: int, K: int) -> str:
    return f"{device_name}|descent|W={int(W)}|H={int(H)}|N={int(N)}|K={int(K)}"


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


def lookup(device_name: str, W: int, H: int, N: int, K: int):
    """Cached tile width for this shape, or None."""
    with _lock:
        e = _load().get(key(device_name, W, H, N, K))
    return int(e["tile_x"]) if e else None


def lookup_leaf(device_name: str, W: int, H: int, N: int, K: int):
    """Cached (tile_x, leaf_size) of a tile x leaf sweep for this shape, or
    None."""
    with _lock:
        e = _load().get(key(device_name, W, H, N, K) + "|leaf")
    return (int(e["tile_x"]), int(e["leaf_size"])) if e else None


def record(device_name: str, W: int, H: int, N: int, K: int, tile_x: int, timings_ms: dict,
           leaf_size=None) -> None:
    with _lock:
        c = _load()
        entry = {"tile_x": int(tile_x), "ms": {str(k): float(v) for k, v in timings_ms.items()}}
        k = key(device_name, W, H, N, K)
        if leaf_size is not None:
            entry["leaf_size"] = int(leaf_size)
            k += "|leaf"
        c[k] = entry
        path = cache_path()
        os.makedirs(os.path.dirname(path), exist_ok=True)
        tmp = path + f".tmp{os.getpid()}"
        with open(tmp, "w") as f:
            json.dump(c, f, indent=1, sort_keys=True)
        os.replace(tmp, path)


def choose(timings_ms: dict) -> int:
    """Fastest candidate (ties: the smaller tile)."""
    return min(sorted(timings_ms), key=lambda t: timings_ms[t])


def tune_descent(width, height, focallength, points, normals, stdDevs, numSamples, smoothing, precision,
                 view=0, reps=3, candidates=CANDIDATES, timer=None, save=True, leaf_sizes=None):
    """Time the descent of view `view` for each candidate tile width and cache
    the fastest.  `timer(tile_x) -> ms` replaces the GPU timing (tests).
    Returns (best tile_x, {tile_x: ms}).

    With `leaf_sizes` (e.g. LEAF_CANDIDATES) every (tile_x, leaf_size) pair is
    timed, `timer(tile_x, leaf_size)`, and the fastest pair is cached for
    ``lookup_leaf``; returns ((tile_x, leaf_size), {"tile/leaf": ms})."""
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

        def timer(tx, leaf=0):
            prm.tile_x = tx
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
    if leaf_sizes is not None:
        pairs = {(int(t), int(lf)): float(timer(int(t), int(lf))) for t in candidates for lf in leaf_sizes}
        tb, lb = min(sorted(pairs), key=lambda q: pairs[q])
        timings = {f"{t}/{lf}": v for (t, lf), v in pairs.items()}
        if save:
            record(name, W, H, N, K, tb, timings, leaf_size=lb)
        return (tb, lb), timings
    timings = {int(t): float(timer(int(t))) for t in candidates}
    best = choose(timings)
    if save:
        record(name, W, H, N, K, best, timings)
    return best, timings
