"""Autotuner cache logic (no GPU: the timing is replaced by a fake timer)."""
import json

import torch

from unbiased_differentiable_splatting_gb300 import autotune


def test_tune_records_fastest(tmp_path, monkeypatch):
    monkeypatch.setenv("UDS_AUTOTUNE_CACHE", str(tmp_path / "cache.json"))
    autotune.reset()
    times = {4: 3.0, 8: 2.0, 16: 2.5, 32: 4.0}
    pts = torch.zeros((1, 1234, 3))
    best, t = autotune.tune_descent(64, 48, 50.0, pts, pts, torch.zeros((1, 1234, 2)), 8, 0.0, 0.01,
                                    timer=lambda tx: times[tx])
    assert best == 8 and t == {k: float(v) for k, v in times.items()}
    assert autotune.lookup("test-device", 64, 48, 1234, 8) == 8
    assert autotune.lookup("test-device", 64, 48, 1235, 8) is None
    data = json.load(open(tmp_path / "cache.json"))
    assert data[autotune.key("test-device", 64, 48, 1234, 8)]["tile_x"] == 8
    # a fresh process (in-memory copy dropped) reads the file back
    autotune.reset()
    assert autotune.lookup("test-device", 64, 48, 1234, 8) == 8
    autotune.reset()


def test_choose_ties_prefer_smaller_tile():
    assert autotune.choose({16: 1.0, 4: 1.0, 8: 2.0}) == 4


def test_tile_leaf_sweep_kept_apart(tmp_path, monkeypatch):
    """The tile x leaf sweep caches its pair under its own entry: the tile-only
    lookup (which never changes the sampled indices) does not see it."""
    monkeypatch.setenv("UDS_AUTOTUNE_CACHE", str(tmp_path / "cache.json"))
    autotune.reset()
    pts = torch.zeros((1, 500, 3))
    cost = {4: 1.3, 8: 1.0, 16: 1.1, 32: 1.6}
    lcost = {0: 1.0, 16: 0.94, 32: 0.99}
    (tile, leaf), t = autotune.tune_descent(32, 32, 30.0, pts, pts, torch.zeros((1, 500, 2)), 8, 0.0, 0.01,
                                            timer=lambda tx, lf: cost[tx] * lcost[lf],
                                            leaf_sizes=autotune.LEAF_CANDIDATES)
    assert (tile, leaf) == (8, 16) and len(t) == len(autotune.CANDIDATES) * len(autotune.LEAF_CANDIDATES)
    assert autotune.lookup_leaf("test-device", 32, 32, 500, 8) == (8, 16)
    assert autotune.lookup("test-device", 32, 32, 500, 8) is None
    autotune.reset()
    assert autotune.lookup_leaf("test-device", 32, 32, 500, 8) == (8, 16)
    autotune.reset()
