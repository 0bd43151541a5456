"""Autotuner cache logic (no GPU: the timing is replaced by a fake timer)."""
import json

import torch

from unbiased_differentiable_splatting_gb300 import autotune


def test_tune_records_fastest(tmp_path, monkeypatch):
    monkeypatch.setenv("UDS_AUTOTUNE_CACHE", str(tmp_path / "cache.json"))
    autotune.reset()
    times = {4: 3.0, 8: 2.0, 16: 2.5, 32: 4.0}
    spread_cost = {0: 1.0, 1: 0.9}
    pts = torch.zeros((1, 1234, 3))
    best, t = autotune.tune_descent(64, 48, 50.0, pts, pts, torch.zeros((1, 1234, 2)), 8, 0.0, 0.01,
                                    timer=lambda tx, sp, lf: times[tx] * spread_cost[sp])
    assert best == {"tile_x": 8, "spread": 1}
    assert t == {f"{tx}/{sp}": times[tx] * spread_cost[sp] for tx in times for sp in spread_cost}
    assert autotune.lookup("test-device", 64, 48, 1234, 8) == 8
    assert autotune.lookup_config("test-device", 64, 48, 1234, 8) == {"tile_x": 8, "spread": 1}
    assert autotune.lookup("test-device", 64, 48, 1235, 8) is None
    data = json.load(open(tmp_path / "cache.json"))
    assert data[autotune.key("test-device", 64, 48, 1234, 8)]["tile_x"] == 8
    # a fresh process (in-memory copy dropped) reads the file back
    autotune.reset()
    assert autotune.lookup_config("test-device", 64, 48, 1234, 8) == {"tile_x": 8, "spread": 1}
    autotune.reset()


def test_choose_ties_prefer_smaller_tile():
    assert autotune.choose({16: 1.0, 4: 1.0, 8: 2.0}) == 4


def test_tile_leaf_sweep_kept_apart(tmp_path, monkeypatch):
    """The sweep with leaf sizes caches its configuration under its own entry:
    the plain lookup (whose choices never change the sampled indices) does
    not see it."""
    monkeypatch.setenv("UDS_AUTOTUNE_CACHE", str(tmp_path / "cache.json"))
    autotune.reset()
    pts = torch.zeros((1, 500, 3))
    cost = {4: 1.3, 8: 1.0, 16: 1.1, 32: 1.6}
    lcost = {0: 1.0, 16: 0.94, 32: 0.99}
    best, t = autotune.tune_descent(32, 32, 30.0, pts, pts, torch.zeros((1, 500, 2)), 8, 0.0, 0.01,
                                    timer=lambda tx, sp, lf: cost[tx] * lcost[lf] * (1.0 + 0.01 * sp),
                                    leaf_sizes=autotune.LEAF_CANDIDATES)
    assert best == {"tile_x": 8, "spread": 0, "leaf_size": 16}
    assert len(t) == len(autotune.CANDIDATES) * len(autotune.SPREADS) * len(autotune.LEAF_CANDIDATES)
    assert autotune.lookup_leaf("test-device", 32, 32, 500, 8) == (8, 16)
    assert autotune.lookup("test-device", 32, 32, 500, 8) is None
    autotune.reset()
    assert autotune.lookup_leaf("test-device", 32, 32, 500, 8) == (8, 16)
    autotune.reset()


def test_views_sweep_keyed_by_view_sizes(tmp_path, monkeypatch):
    monkeypatch.setenv("UDS_AUTOTUNE_CACHE", str(tmp_path / "cache.json"))
    autotune.reset()
    pts = torch.zeros((2, 300, 3))
    views = [(64, 48, 50.0), (32, 32, 30.0)]
    best, t = autotune.tune_views(views, pts, pts, torch.zeros((1, 300, 2)), 8, 0.0, 0.01,
                                  timer=lambda tx, sp, lf: {4: 2.0, 8: 1.5, 16: 1.7, 32: 3.0}[tx] + 0.1 * sp)
    assert best == {"tile_x": 8, "spread": 0}
    assert autotune.lookup_views("test-device", views, 300, 8) == best
    assert autotune.lookup_views("test-device", views[::-1], 300, 8) is None
    assert autotune.lookup("test-device", 64, 48, 300, 8) is None
    autotune.reset()


def test_sampler_resolves_cached_configuration(tmp_path, monkeypatch):
    """sampling._descent / _descent_views take the given values first, then
    the cached configuration for the shape (or list of views), then the
    defaults; leaf_size="auto" reads only the sweep with leaf sizes."""
    from unbiased_differentiable_splatting_gb300.cudaExtensions import sampling
    monkeypatch.setenv("UDS_AUTOTUNE_CACHE", str(tmp_path / "cache.json"))
    monkeypatch.setitem(sampling._device_names, None, "test-device")  # CPU tensors: device index None
    autotune.reset()
    pts = torch.zeros((1, 700, 3))
    assert sampling._descent(pts, 64, 48, 8) == (8, 0, 0)  # nothing cached: defaults
    autotune.record("test-device", 64, 48, 700, 8, {"tile_x": 16, "spread": 1}, {})
    assert sampling._descent(pts, 64, 48, 8) == (16, 0, 1)
    assert sampling._descent(pts, 64, 48, 8, tile_x=4) == (4, 0, 1)
    assert sampling._descent(pts, 64, 48, 8, spread=0) == (16, 0, 0)
    assert sampling._descent(pts, 64, 48, 8, leaf_size=32) == (16, 32, 1)
    assert sampling._descent(pts, 64, 48, 8, leaf_size="auto") == (16, 0, 1)  # no leaf sweep cached
    autotune.record("test-device", 64, 48, 700, 8, {"tile_x": 4, "spread": 0, "leaf_size": 16}, {})
    assert sampling._descent(pts, 64, 48, 8, leaf_size="auto") == (4, 16, 0)
    assert sampling._descent(pts, 64, 48, 8) == (16, 0, 1)  # the plain entry is unchanged
    views = [(64, 48, 50.0), (32, 32, 30.0)]
    assert sampling._descent_views(views, pts, 8) == (16, 0, 1)  # falls back to the first view's shape
    autotune.record("test-device", 0, 0, 700, 8, {"tile_x": 32, "spread": 0}, {}, views=views)
    assert sampling._descent_views(views, pts, 8) == (32, 0, 0)
    assert sampling._descent_views(views, pts, 8, tile_x=8, spread=1) == (8, 0, 1)
    autotune.reset()
