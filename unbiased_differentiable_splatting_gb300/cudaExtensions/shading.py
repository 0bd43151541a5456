"""cudaExtensions.shading (shading.cpp:51-199): deferred Lambert and
order-2 spherical-harmonics shading of per-pixel normals and albedo; and the
fused per-splat Lambert of the forward shading mode (shading.py:12-29)."""
from __future__ import annotations

import torch

from .._lib import check, load, need, ptr, stream_ptr


def _pix(normals, diffuse):
    need(normals, "normals")
    need(diffuse, "diffuse", device=normals.device)
    if normals.shape != diffuse.shape or normals.shape[-1] != 3:
        raise ValueError("normals and diffuse must both be (B,W,H,3)")
    B = normals.shape[0]
    return B, normals.numel() // (3 * B)


def forward(directions, intensities, normals, diffuse):
    B, P = _pix(normals, diffuse)
    need(directions, "directions", device=normals.device)
    need(intensities, "intensities", device=normals.device)
    L = intensities.shape[1]
    out = torch.empty_like(normals)
    check(load().uds_shade_forward(B, P, L, ptr(directions), ptr(intensities), intensities.shape[0], ptr(normals),
                                   ptr(diffuse), ptr(out), stream_ptr(normals.device)), "shading forward")
    return out


def backward(gradIn, directions, intensities, normals, diffuse):
    B, P = _pix(normals, diffuse)
    need(gradIn, "gradIn", device=normals.device)
    need(directions, "directions", device=normals.device)
    need(intensities, "intensities", device=normals.device)
    L = intensities.shape[1]
    gd, gI = torch.empty_like(directions), torch.empty_like(intensities)
    gn, gdf = torch.empty_like(normals), torch.empty_like(diffuse)
    check(load().uds_shade_backward(B, P, L, ptr(gradIn), ptr(directions), ptr(intensities), intensities.shape[0],
                                    ptr(normals), ptr(diffuse), ptr(gd), ptr(gI), ptr(gn), ptr(gdf),
                                    stream_ptr(normals.device)), "shading backward")
    return [gd, gI, gn, gdf]


def forwardSh(coefficients, normals, diffuse):
    B, P = _pix(normals, diffuse)
    need(coefficients, "coefficients", device=normals.device)
    out = torch.empty_like(normals)
    check(load().uds_shade_sh_forward(B, P, ptr(coefficients), coefficients.shape[0], ptr(normals), ptr(diffuse),
                                      ptr(out), stream_ptr(normals.device)), "shading forwardSh")
    return out


def backwardSh(gradIn, coefficients, normals, diffuse):
    B, P = _pix(normals, diffuse)
    need(gradIn, "gradIn", device=normals.device)
    need(coefficients, "coefficients", device=normals.device)
    gc, gn, gd = torch.empty_like(coefficients), torch.empty_like(normals), torch.empty_like(diffuse)
    check(load().uds_shade_sh_backward(B, P, ptr(gradIn), ptr(coefficients), coefficients.shape[0], ptr(normals),
                                       ptr(diffuse), ptr(gc), ptr(gn), ptr(gd), stream_ptr(normals.device)),
          "shading backwardSh")
    return [gc, gn, gd]


LAMBERT_MAX_LIGHTS = 4


def lambert_shapes(ambient, directions, intensities, normals, diffuse):
    """(B, N, L, aB, IB, dB) when the operands have the shapes the fused
    kernel takes, else None: normals (B, N, 3), diffuse (dB, N, 3), directions
    (B, L, 3), intensities (IB, L, 3), ambient (aB, 1, 3) with aB in {1, B},
    or (1, 3) or (3,); dB, IB in {1, B}; float32 CUDA tensors on one device.
    A 2-D ambient with more than one row broadcasts against the splat axis in
    the reference's expression ``ambientLight * diffuse`` (one ambient per
    splat when it has N rows, an error otherwise), so it is left to that
    expression."""
    ts = (ambient, directions, intensities, normals, diffuse)
    if not all(isinstance(t, torch.Tensor) and t.is_cuda and t.dtype == torch.float32 for t in ts):
        return None
    if len({t.device for t in ts}) != 1 or normals.dim() != 3 or normals.shape[-1] != 3:
        return None
    B, N = normals.shape[0], normals.shape[1]
    if directions.dim() != 3 or directions.shape[0] != B or directions.shape[2] != 3:
        return None
    L = directions.shape[1]
    if L > LAMBERT_MAX_LIGHTS or intensities.dim() != 3 or tuple(intensities.shape[1:]) != (L, 3):
        return None
    if diffuse.dim() != 3 or tuple(diffuse.shape[1:]) != (N, 3):
        return None
    IB, dB = intensities.shape[0], diffuse.shape[0]
    if ambient.shape[-1] != 3 or ambient.dim() > 3:
        return None
    if ambient.dim() == 3:
        if ambient.shape[1] != 1:
            return None
        aB = ambient.shape[0]
    else:
        if ambient.dim() == 2 and ambient.shape[0] != 1:
            return None
        aB = 1
    if any(x not in (1, B) for x in (IB, dB, aB)):
        return None
    return B, N, L, aB, IB, dB


def lambertForward(ambient, directions, intensities, normals, diffuse):
    B, N, L, aB, IB, dB = lambert_shapes(ambient, directions, intensities, normals, diffuse)
    out = torch.empty_like(normals)
    check(load().uds_lambert_forward(B, N, L, ptr(ambient), aB, ptr(directions), ptr(intensities), IB,
                                     ptr(normals), ptr(diffuse), dB, ptr(out), stream_ptr(normals.device)),
          "lambert forward")
    return out


def lambertBackward(gradIn, ambient, directions, intensities, normals, diffuse):
    B, N, L, aB, IB, dB = lambert_shapes(ambient, directions, intensities, normals, diffuse)
    need(gradIn, "gradIn", device=normals.device)
    ga, gdir, gI = torch.empty_like(ambient), torch.empty_like(directions), torch.empty_like(intensities)
    gn, gd = torch.empty_like(normals), torch.empty_like(diffuse)
    check(load().uds_lambert_backward(B, N, L, ptr(gradIn), ptr(ambient), aB, ptr(directions), ptr(intensities),
                                      IB, ptr(normals), ptr(diffuse), dB, ptr(ga), ptr(gdir), ptr(gI), ptr(gn),
                                      ptr(gd), stream_ptr(normals.device)), "lambert backward")
    return [ga, gdir, gI, gn, gd]
