"""cudaExtensions.shading (shading.cpp:51-199): deferred Lambert and
order-2 spherical-harmonics shading of per-pixel normals and albedo."""
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
