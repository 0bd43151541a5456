"""Scene file formats (no GPU)."""
import json
import struct

import numpy as np

from unbiased_differentiable_splatting_gb300 import scene_io


def test_ply_round_trip(tmp_path):
    rng = np.random.default_rng(0)
    p = rng.normal(size=(50, 3)).astype(np.float32)
    n = rng.normal(size=(50, 3)).astype(np.float32)
    c = rng.uniform(-0.2, 1.2, size=(50, 3))
    f = tmp_path / "a.ply"
    scene_io.write_ply(f, p, n, c)
    v2, n2, c2 = scene_io.read_ply(f)
    np.testing.assert_array_equal(v2, p)
    np.testing.assert_array_equal(n2, n)
    np.testing.assert_allclose(c2, (np.clip(c, 0, 1) * 255).astype(np.int64) / 255.0, rtol=1e-6)


def test_ply_ascii_without_colors(tmp_path):
    f = tmp_path / "b.ply"
    f.write_text("ply\nformat ascii 1.0\ncomment x\nelement vertex 2\nproperty double nx\nproperty double ny\n"
                 "property double nz\nproperty float x\nproperty float y\nproperty float z\nend_header\n"
                 "0 0 1 1 2 3\n1 0 0 4 5 6\n")
    v, n, c = scene_io.read_ply(f)
    np.testing.assert_array_equal(v, [[1, 2, 3], [4, 5, 6]])
    np.testing.assert_array_equal(n, [[0, 0, 1], [1, 0, 0]])
    assert np.all(c == 1.0)


def test_poses_and_frames(tmp_path):
    ms = [np.arange(16, dtype=np.float32).reshape(4, 4) + i for i in range(3)]
    scene_io.write_poses(tmp_path / "pose.dat", ms, frames=[7, 8, 9])
    raw = (tmp_path / "pose.dat").read_bytes()
    assert len(raw) == 216 and struct.unpack_from("<q", raw, 72)[0] == 8
    back = scene_io.read_poses(tmp_path / "pose.dat")
    for a, b in zip(ms, back):
        np.testing.assert_array_equal(a, b)
    (tmp_path / "rgb.txt").write_text("# comment\n2.5 rgb/b.png\n1.0 rgb/a.png\n")
    assert scene_io.read_frame_list(str(tmp_path), "rgb.txt") == [str(tmp_path / "rgb/a.png"),
                                                                   str(tmp_path / "rgb/b.png")]


def test_calibration_and_lighting(tmp_path):
    (tmp_path / "calibration.yml").write_text(
        "%YAML:1.0\n# camera\ncalibration_geometric:\n  intrinsics_color:\n    focal_lengths:\n      x: 525.0\n      y: 525.0\n"
        "    resolution:\n      x: 640\n      y: 480\n  extra: 'abc'\nrange:\n  min: 0.1   # metres\n  max: 10\n")
    assert scene_io.read_calibration(tmp_path / "calibration.yml") == (640, 480, 525.0, 0.1, 10)
    (tmp_path / "lights.json").write_text(json.dumps({"Ambient": [0.1, 0.2, 0.3],
                                                      "Lights": [{"Direction": [0, 0, 2], "Color": [1, 1, 1]}]}))
    amb, d, c = scene_io.read_lighting(tmp_path / "lights.json")
    assert amb.shape == (1, 1, 3) and d.shape == (1, 1, 3) and abs(float(d[0, 0, 2]) - 2 / 2.0001) < 1e-6
    np.testing.assert_allclose(c, np.pi, rtol=1e-6)
