"""Scene file formats of the reference's datasets (splatting/dataset.py),
read and written without third-party packages:

* ``read_ply`` / ``write_ply``: point sets with positions, normals and 8-bit
  colours (dataset.py:100-147; ``binary_little_endian`` or ``ascii`` PLY,
  vertex properties in any order and of any PLY scalar type; colours default
  to white as in the reference);
* ``read_poses``: ``pose.dat``, 72-byte records of an 8-byte little-endian
  frame number and a row-major 4x4 float32 matrix (dataset.py:77-86);
* ``read_frame_list``: ``rgb.txt`` / ``depth.txt``, ``timestamp filename``
  lines sorted by timestamp, ``#`` comments (dataset.py:88-98);
* ``read_calibration``: ``calibration.yml`` -> (width, height, focal length,
  zmin, zmax) (dataset.py:149-162), with a parser for the block-mapping subset
  of YAML these files use;
* ``read_lighting``: ``lights.json`` -> (ambient (1,1,3), directions (1,L,3),
  intensities (1,L,3)) (dataset.py:44-60).
"""
from __future__ import annotations

import json
import math
import os
import struct

import numpy as np

_PLY_TYPES = {"char": "i1", "int8": "i1", "uchar": "u1", "uint8": "u1", "short": "i2", "int16": "i2",
              "ushort": "u2", "uint16": "u2", "int": "i4", "int32": "i4", "uint": "u4", "uint32": "u4",
              "float": "f4", "float32": "f4", "double": "f8", "float64": "f8"}


def read_ply(path):
    """(vertices (N,3), normals (N,3), colors (N,3) in [0,1]) as float32."""
    with open(path, "rb") as f:
        if f.readline().strip() != b"ply":
            raise ValueError(f"{path}: not a PLY file")
        fmt, elements, cur = None, [], None
        while True:
            line = f.readline()
            if not line:
                raise ValueError(f"{path}: PLY header without end_header")
            tok = line.decode("ascii", "replace").split()
            if not tok or tok[0] in ("comment", "obj_info"):
                continue
            if tok[0] == "format":
                fmt = tok[1]
            elif tok[0] == "element":
                cur = {"name": tok[1], "count": int(tok[2]), "props": []}
                elements.append(cur)
            elif tok[0] == "property":
                if tok[1] == "list":
                    cur["props"].append((tok[4], "list", tok[2], tok[3]))
                else:
                    cur["props"].append((tok[2], tok[1]))
            elif tok[0] == "end_header":
                break
        if not elements or elements[0]["name"] != "vertex":
            raise ValueError(f"{path}: the first PLY element must be 'vertex'")
        vert = elements[0]
        if any(p[1] == "list" for p in vert["props"]):
            raise ValueError(f"{path}: list properties on vertices are not supported")
        names = [p[0] for p in vert["props"]]
        if fmt == "binary_little_endian" or fmt == "binary_big_endian":
            end = "<" if fmt == "binary_little_endian" else ">"
            dt = np.dtype([(p[0], end + _PLY_TYPES[p[1]]) for p in vert["props"]])
            data = np.frombuffer(f.read(dt.itemsize * vert["count"]), dtype=dt, count=vert["count"])
            col = {n: data[n].astype(np.float64) for n in names}
        elif fmt == "ascii":
            rows = [f.readline().split() for _ in range(vert["count"])]
            arr = np.array(rows, dtype=np.float64).reshape(vert["count"], len(names))
            col = {n: arr[:, i] for i, n in enumerate(names)}
        else:
            raise ValueError(f"{path}: unsupported PLY format {fmt}")
    v = np.stack([col["x"], col["y"], col["z"]], -1).astype(np.float32)
    n = np.stack([col["nx"], col["ny"], col["nz"]], -1).astype(np.float32)
    if all(k in col for k in ("red", "green", "blue")):
        c = np.stack([col["red"], col["green"], col["blue"]], -1).astype(np.float32)
    else:
        c = np.full_like(n, 255.0)
    return v, n, c / 255.0


def write_ply(path, points, normals, colors):
    """The reference's PLY layout (dataset.py:112-139): binary little-endian
    float x y z nx ny nz, uchar red green blue alpha (alpha 1), colours
    clamped to [0,1] and truncated to 8 bits, an empty face element."""
    points = np.asarray(points, np.float32).reshape(-1, 3)
    normals = np.asarray(normals, np.float32).reshape(-1, 3)
    colors = np.asarray(colors, np.float64).reshape(-1, 3)
    header = ("ply\nformat binary_little_endian 1.0\ncomment VCGLIB generated\n"
              f"element vertex {len(points)}\n"
              "property float x\nproperty float y\nproperty float z\n"
              "property float nx\nproperty float ny\nproperty float nz\n"
              "property uchar red\nproperty uchar green\nproperty uchar blue\nproperty uchar alpha\n"
              "element face 0\nproperty list uchar int vertex_indices\nend_header\n")
    dt = np.dtype([("p", "<f4", 3), ("n", "<f4", 3), ("c", "u1", 4)])
    rec = np.zeros(len(points), dtype=dt)
    rec["p"] = points
    rec["n"] = normals
    rec["c"][:, :3] = (np.clip(colors, 0.0, 1.0) * 255).astype(np.int64)
    rec["c"][:, 3] = 1
    with open(path, "wb") as f:
        f.write(header.encode("ascii"))
        f.write(rec.tobytes())


def read_poses(path, dtype=np.float32):
    """List of 4x4 matrices from 72-byte records (frame number ignored, as in
    the reference)."""
    raw = open(path, "rb").read()
    if len(raw) % 72:
        raise ValueError(f"{path}: size {len(raw)} is not a multiple of 72")
    out = []
    for o in range(0, len(raw), 72):
        m = np.array(struct.unpack_from("<16f", raw, o + 8), dtype=np.float64).reshape(4, 4)
        out.append(m.astype(dtype))
    return out


def write_poses(path, matrices, frames=None):
    with open(path, "wb") as f:
        for i, m in enumerate(matrices):
            f.write(struct.pack("<q", int(frames[i]) if frames is not None else i))
            f.write(struct.pack("<16f", *np.asarray(m, np.float32).reshape(16).tolist()))


def read_frame_list(root, framelist):
    """Frame paths of ``framelist`` (``timestamp filename`` per line) sorted
    by timestamp."""
    entries = []
    with open(os.path.join(root, framelist)) as f:
        for line in f:
            if not line.strip() or line[0] == "#":
                continue
            ts, name = line.rstrip("\n").split(" ", 1)
            entries.append((float(ts), name))
    entries.sort(key=lambda e: e[0])
    return [os.path.join(root, n) for _, n in entries]


def _scalar(s):
    s = s.strip()
    if s and s[0] in "'\"" and s[-1] == s[0]:
        return s[1:-1]
    low = s.lower()
    if low in ("true", "false"):
        return low == "true"
    if low in ("null", "~", ""):
        return None
    try:
        return int(s)
    except ValueError:
        pass
    try:
        return float(s)
    except ValueError:
        return s


def parse_yaml_mapping(text):
    """Nested block mappings (``key: value`` / ``key:`` + indented block),
    comments and scalars; enough for calibration.yml."""
    root = {}
    stack = [(-1, root)]
    for raw in text.splitlines():
        line = raw.split(" #", 1)[0].rstrip() if not raw.lstrip().startswith("#") else ""
        if not line.strip() or line.strip() in ("---", "...") or line.startswith("%"):
            continue  # blank, document markers, directives (%YAML:1.0)
        indent = len(line) - len(line.lstrip(" "))
        key, sep, val = line.strip().partition(":")
        if not sep:
            raise ValueError(f"unsupported YAML line: {raw!r}")
        while stack[-1][0] >= indent:
            stack.pop()
        parent = stack[-1][1]
        key = _scalar(key)
        if val.strip():
            parent[key] = _scalar(val)
        else:
            parent[key] = {}
            stack.append((indent, parent[key]))
    return root


def read_calibration(path):
    """(width, height, focal length, zmin, zmax) of calibration.yml."""
    meta = parse_yaml_mapping(open(path).read())
    cal = meta["calibration_geometric"]["intrinsics_color"]
    fl = cal["focal_lengths"]
    if fl["x"] != fl["y"]:
        raise ValueError("focal lengths differ in x and y")
    res = cal["resolution"]
    rng = meta["range"]
    return res["x"], res["y"], fl["x"], rng["min"], rng["max"]


def read_lighting(path):
    """lights.json -> ambient (1,1,3), unit directions (1,L,3), intensities
    pi * colour (1,L,3) (no lights: one zero light along +z)."""
    d = json.load(open(path))
    amb = np.asarray(d["Ambient"], np.float32).reshape(1, 1, 3)
    lights = d["Lights"]
    if lights:
        dirs = np.asarray([l["Direction"] for l in lights], np.float32).reshape(1, -1, 3)
        cols = (math.pi * np.asarray([l["Color"] for l in lights], np.float32)).reshape(1, -1, 3)
    else:
        dirs = np.array([[[0.0, 0.0, 1.0]]], np.float32)
        cols = np.zeros((1, 1, 3), np.float32)
    dirs = dirs / (np.linalg.norm(dirs, axis=-1, keepdims=True) + 1e-4)
    return amb, dirs.astype(np.float32), cols.astype(np.float32)
