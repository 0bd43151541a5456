"""Seeded synthetic scenes with the shapes, sizes and value distributions of the
five benchmark workloads (no datasets are available offline).

Every generator returns a dict of float32 torch tensors on the CPU:
``points, normals (1,N,3)``, ``stddevs (1,N,2)``, ``colors (1,N,C)``,
``cam_positions (B,3)``, ``cam_orientations (B,4)`` (quaternion x,y,z,w for
``world2Camera`` with forward '-z'), ``lamp_directions (B,L,3)``,
``lamp_intensities (1,L,3)``, ``ambient (1,1,3)``, and the image size and
focal length.  Camera space looks down -z, like the reference's sampler
expects (visible splats have z <= 0).
"""
from __future__ import annotations

import math

import numpy as np
import torch
from scipy.special import lpmv


def focal_from_fov(width: int, fov_deg: float = 60.0) -> float:
    return (width / 2.0) / math.tan(math.radians(fov_deg) / 2.0)


def _t(a):
    return torch.from_numpy(np.ascontiguousarray(a, dtype=np.float32))


def _unit_directions(rng, n):
    v = rng.normal(size=(n, 3))
    return v / np.linalg.norm(v, axis=1, keepdims=True)


def _front_camera(distance: float, B: int = 1):
    # world -> camera = identity rotation + translation (0, 0, -distance)
    return _t(np.tile([[0.0, 0.0, -distance]], (B, 1))), _t(np.tile([[0.0, 0.0, 0.0, 1.0]], (B, 1)))


def _lights(B: int, L: int = 1):
    d = np.array([0.3, 0.4, 1.0])
    d /= np.linalg.norm(d)
    return _t(np.tile(d, (B, L, 1))), _t(np.ones((1, L, 3))), _t(np.full((1, 1, 3), 0.1))


def sphere_scene(n=4096, radius=0.5, jitter=0.01, sd=0.005, width=128, seed=0):
    """4,096 surfels uniform on a sphere of radius 0.5 with N(0, 0.01) radial
    jitter, radial normals, RGB in U[0,1], isotropic std-dev 0.005; camera at
    distance 2, 60 deg fov, 128x128."""
    rng = np.random.default_rng(seed)
    d = _unit_directions(rng, n)
    r = radius + rng.normal(0.0, jitter, size=(n, 1))
    cp, co = _front_camera(2.0)
    ld, li, amb = _lights(1)
    return dict(points=_t(d * r)[None], normals=_t(d)[None], stddevs=_t(np.full((n, 2), sd))[None],
                colors=_t(rng.uniform(0, 1, size=(n, 3)))[None], cam_positions=cp, cam_orientations=co,
                lamp_directions=ld, lamp_intensities=li, ambient=amb, width=width, height=width,
                focal=focal_from_fov(width))


def _real_sh(l, m, theta, phi):
    am = abs(m)
    norm = math.sqrt((2 * l + 1) / (4 * math.pi) * math.factorial(l - am) / math.factorial(l + am))
    p = lpmv(am, l, np.cos(theta))
    if m > 0:
        return math.sqrt(2) * norm * p * np.cos(am * phi)
    if m < 0:
        return math.sqrt(2) * norm * p * np.sin(am * phi)
    return norm * p


def harmonic_surface(n, rng, base=0.6, amp=0.2, terms=4, max_l=4):
    """Star-shaped surface r(theta, phi) = base (1 + amp * sum of `terms`
    random real spherical harmonics of degree <= max_l), normals from the
    parametric surface."""
    ls = rng.integers(1, max_l + 1, size=terms)
    ms = [int(rng.integers(-l, l + 1)) for l in ls]
    ws = rng.uniform(-1.0, 1.0, size=terms)

    def radius(th, ph):
        s = sum(w * _real_sh(int(l), m, th, ph) for w, l, m in zip(ws, ls, ms))
        return base * (1.0 + amp * s)

    def surf(th, ph):
        r = radius(th, ph)
        return np.stack([r * np.sin(th) * np.cos(ph), r * np.sin(th) * np.sin(ph), r * np.cos(th)], -1)

    d = _unit_directions(rng, n)
    th = np.arccos(np.clip(d[:, 2], -1, 1))
    th = np.clip(th, 1e-3, math.pi - 1e-3)
    ph = np.arctan2(d[:, 1], d[:, 0])
    P = surf(th, ph)
    e = 1e-5
    dth = (surf(th + e, ph) - surf(th - e, ph)) / (2 * e)
    dph = (surf(th, ph + e) - surf(th, ph - e)) / (2 * e)
    nrm = np.cross(dth, dph)
    nrm /= np.linalg.norm(nrm, axis=1, keepdims=True) + 1e-12
    flip = np.sum(nrm * P, axis=1) < 0
    nrm[flip] *= -1.0
    return P, nrm


def harmonic_scene(n=100_000, sd_range=(0.0045, 0.009), width=512, seed=0, albedo=(0.2, 0.9), channels=3):
    """Single-view shape-optimisation workload: surfels on a random-harmonic
    star-shaped surface, per-axis std-devs uniform in sd_range, albedo uniform
    in `albedo`, one directional light (100k / 512^2; 500k / 1024^2 with
    sd_range (0.003, 0.01))."""
    rng = np.random.default_rng(seed)
    P, nrm = harmonic_surface(n, rng)
    sd = rng.uniform(sd_range[0], sd_range[1], size=(n, 2))
    col = rng.uniform(albedo[0], albedo[1], size=(n, channels))
    cp, co = _front_camera(2.0)
    ld, li, amb = _lights(1)
    return dict(points=_t(P)[None], normals=_t(nrm)[None], stddevs=_t(sd)[None], colors=_t(col)[None],
                cam_positions=cp, cam_orientations=co, lamp_directions=ld, lamp_intensities=li, ambient=amb,
                width=width, height=width, focal=focal_from_fov(width))


def feature_scene(n=300_000, channels=8, sd=0.005, seed=0):
    """Uneven-batch workload cloud: harmonic surface, `channels` N(0,1)
    features per surfel, isotropic std-dev."""
    rng = np.random.default_rng(seed)
    P, nrm = harmonic_surface(n, rng)
    return dict(points=_t(P)[None], normals=_t(nrm)[None], stddevs=_t(np.full((n, 2), sd))[None],
                colors=_t(rng.normal(size=(n, channels)))[None])


def _quat_look(forward_cam_to_world: np.ndarray, up=np.array([0.0, 0.0, 1.0])):
    """Quaternion (x,y,z,w) of the world->camera rotation whose camera looks
    along `forward` (camera -z) with the given up vector."""
    f = forward_cam_to_world / np.linalg.norm(forward_cam_to_world)
    r = np.cross(f, up)
    if np.linalg.norm(r) < 1e-6:
        r = np.cross(f, np.array([0.0, 1.0, 0.0]))
    r /= np.linalg.norm(r)
    u = np.cross(r, f)
    Rw = np.stack([r, u, -f], 0)  # rows: camera axes in world
    m = Rw
    t = np.trace(m)
    if t > 0:
        s = math.sqrt(t + 1.0) * 2
        w = 0.25 * s
        x = (m[2, 1] - m[1, 2]) / s
        y = (m[0, 2] - m[2, 0]) / s
        z = (m[1, 0] - m[0, 1]) / s
    else:
        i = int(np.argmax(np.diag(m)))
        j, k = (i + 1) % 3, (i + 2) % 3
        s = math.sqrt(1.0 + m[i, i] - m[j, j] - m[k, k]) * 2
        q = np.zeros(4)
        q[i] = 0.25 * s
        q[3] = (m[k, j] - m[j, k]) / s
        q[j] = (m[j, i] + m[i, j]) / s
        q[k] = (m[k, i] + m[i, k]) / s
        x, y, z, w = q
    return np.array([x, y, z, w]), Rw


def room_scene(n=2_000_000, views=16, width=640, height=480, focal=525.0, n_boxes=40, sd_range=(0.005, 0.02),
               seed=0):
    """Pose + scene refinement workload: surfels on the inner walls of a
    5 x 5 x 3 m room and on 40 random boxes, std-devs in sd_range, `views`
    cameras at random interior poses looking at random wall points."""
    rng = np.random.default_rng(seed)
    # area-weighted split between room faces and box faces
    faces = []  # (origin, u, v, inward normal)
    Lx, Ly, Lz = 5.0, 5.0, 3.0
    faces += [((0, 0, 0), (Lx, 0, 0), (0, Ly, 0), (0, 0, 1)), ((0, 0, Lz), (Lx, 0, 0), (0, Ly, 0), (0, 0, -1)),
              ((0, 0, 0), (Lx, 0, 0), (0, 0, Lz), (0, 1, 0)), ((0, Ly, 0), (Lx, 0, 0), (0, 0, Lz), (0, -1, 0)),
              ((0, 0, 0), (0, Ly, 0), (0, 0, Lz), (1, 0, 0)), ((Lx, 0, 0), (0, Ly, 0), (0, 0, Lz), (-1, 0, 0))]
    for _ in range(n_boxes):
        size = rng.uniform(0.2, 0.8, size=3)
        o = np.array([rng.uniform(0.2, Lx - 0.2 - size[0]), rng.uniform(0.2, Ly - 0.2 - size[1]), 0.0])
        sx, sy, sz = size
        faces += [(o + (0, 0, sz), (sx, 0, 0), (0, sy, 0), (0, 0, 1)),
                  (tuple(o), (sx, 0, 0), (0, 0, sz), (0, -1, 0)), (o + (0, sy, 0), (sx, 0, 0), (0, 0, sz), (0, 1, 0)),
                  (tuple(o), (0, sy, 0), (0, 0, sz), (-1, 0, 0)), (o + (sx, 0, 0), (0, sy, 0), (0, 0, sz), (1, 0, 0))]
    area = np.array([np.linalg.norm(np.cross(u, v)) for _, u, v, _ in faces])
    counts = rng.multinomial(n, area / area.sum())
    P, Nn = [], []
    for (o, u, v, nn), c in zip(faces, counts):
        a = rng.uniform(0, 1, size=(c, 2))
        P.append(np.asarray(o) + a[:, :1] * np.asarray(u) + a[:, 1:] * np.asarray(v))
        Nn.append(np.tile(nn, (c, 1)))
    P = np.concatenate(P)
    Nn = np.concatenate(Nn).astype(np.float64)
    sd = rng.uniform(sd_range[0], sd_range[1], size=(n, 2))
    col = rng.uniform(0.2, 0.9, size=(n, 3))
    cams, quats = [], []
    for _ in range(views):
        c = np.array([rng.uniform(1.0, 4.0), rng.uniform(1.0, 4.0), rng.uniform(1.0, 2.0)])
        target = np.array([rng.uniform(0, Lx), rng.uniform(0, Ly), rng.uniform(0.3, 2.7)])
        q, Rw = _quat_look(target - c)
        cams.append(-Rw @ c)  # translation of world -> camera
        quats.append(q)
    ld, li, amb = _lights(views)
    return dict(points=_t(P)[None], normals=_t(Nn)[None], stddevs=_t(sd)[None], colors=_t(col)[None],
                cam_positions=_t(np.array(cams)), cam_orientations=_t(np.array(quats)), lamp_directions=ld,
                lamp_intensities=li, ambient=amb, width=width, height=height, focal=focal)


def orbit_cameras(views: int, distance: float = 2.0, seed: int = 0):
    """`views` cameras at `distance` from the origin in random directions of
    the upper hemisphere (z > 0.2 of the unit direction), each looking at the
    origin: (cam_positions (views,3) world->camera translations,
    cam_orientations (views,4) quaternions)."""
    rng = np.random.default_rng(seed)
    cams, quats = [], []
    while len(cams) < views:
        d = _unit_directions(rng, 1)[0]
        if d[2] < 0.2:
            continue
        c = distance * d
        q, Rw = _quat_look(-c)
        cams.append(-Rw @ c)
        quats.append(q)
    return _t(np.array(cams)), _t(np.array(quats))


def camera_space(scene, device="cpu"):
    """Camera-space points / normals (B,N,3) of a scene (same transform as
    ``Splatting.forward`` for forward '-z'), for calling the ops directly."""
    from .extensions import world2Camera
    M = world2Camera(scene["cam_positions"], scene["cam_orientations"]).squeeze(1)
    R, t = M[:, :3, :3], M[:, :3, 3]
    pts = torch.einsum("bij,nj->bni", R, scene["points"][0]) + t[:, None, :]
    nrm = torch.einsum("bij,nj->bni", R, scene["normals"][0])
    return pts.contiguous().to(device), nrm.contiguous().to(device)
