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
