"""cudaExtensions.splatting (splatting.cpp:43-129)."""
from __future__ import annotations

import torch

from .._lib import Workspace, check, load, need, ptr, stream_ptr


def _check(indices, points, normals, stdDevs):
    need(indices, "indices", torch.int32)
    dev = indices.device
    need(points, "points", device=dev)
    need(normals, "normals", device=dev)
    need(stdDevs, "stdDevs", device=dev)
    if indices.dim() != 4 or points.dim() != 3 or points.shape != normals.shape or stdDevs.dim() != 3:
        raise ValueError("expected indices (B,W,H,K), points/normals (B,N,3), stdDevs (1|B,N,2)")
    B, N = points.shape[0], points.shape[1]
    if indices.shape[0] != B or stdDevs.shape[1] != N or stdDevs.shape[0] not in (1, B):
        raise ValueError("batch / splat counts of indices, points and stdDevs disagree")


def forward(width: int, height: int, focallength: float, indices, points, normals, stdDevs, smoothing: float):
    _check(indices, points, normals, stdDevs)
    B, W, H, K = indices.shape
    if W != width or H != height:
        raise ValueError("indices shape does not match width/height")
    N = points.shape[1]
    L = load()
    nbytes = L.uds_splat_workspace_size(B, N)
    ws = Workspace.get(points.device, nbytes, "splat")
    weights = torch.empty(indices.shape, dtype=torch.float32, device=points.device)
    check(L.uds_splat_forward(B, W, H, K, float(focallength), ptr(indices), ptr(points), ptr(normals),
                              stdDevs.shape[0], N, ptr(stdDevs), float(smoothing), ptr(weights), ptr(ws), ws.numel(),
                              stream_ptr(points.device)), "splatting forward")
    return weights


def backward(width: int, height: int, focallength: float, gradIn, indices, points, normals, stdDevs,
             smoothing: float):
    _check(indices, points, normals, stdDevs)
    need(gradIn, "gradIn", device=points.device)
    B, W, H, K = indices.shape
    if tuple(gradIn.shape) != tuple(indices.shape):
        raise ValueError("gradIn must match indices")
    N = points.shape[1]
    L = load()
    nbytes = L.uds_splat_workspace_size(B, N)
    ws = Workspace.get(points.device, nbytes, "splat")
    gp = torch.empty_like(points)
    gn = torch.empty_like(normals)
    gs = torch.empty_like(stdDevs)
    check(L.uds_splat_backward(B, W, H, K, float(focallength), ptr(gradIn), ptr(indices), ptr(points), ptr(normals),
                               stdDevs.shape[0], N, ptr(stdDevs), float(smoothing), ptr(gp), ptr(gn), ptr(gs), ptr(ws),
                               ws.numel(), stream_ptr(points.device)), "splatting backward")
    return [gp, gn, gs]


def renderForward(width: int, height: int, focallength: float, indices, points, normals, stdDevs, smoothing: float,
                  attribute):
    """splatting.forward -> filtering.forward -> interpolation.forward of
    per-splat attributes (1|B,N,C) in one fused pass (no counterpart module in
    the reference; bit-identical to the three calls).  Returns (image
    (B,W,H,C), depth weights (B,W,H,K), EWA weights (B,W,H,K))."""
    _check(indices, points, normals, stdDevs)
    need(attribute, "attribute", device=points.device)
    B, W, H, K = indices.shape
    if W != width or H != height:
        raise ValueError("indices shape does not match width/height")
    N = points.shape[1]
    if attribute.dim() != 3 or attribute.shape[1] != N or attribute.shape[0] not in (1, B):
        raise ValueError("attribute must be (1|B,N,C)")
    C = attribute.shape[2]
    L = load()
    ws = Workspace.get(points.device, L.uds_splat_workspace_size(B, N), "splat")
    weights = torch.empty(indices.shape, dtype=torch.float32, device=points.device)
    depth = torch.empty_like(weights)
    image = torch.empty((B, W, H, C), dtype=torch.float32, device=points.device)
    check(L.uds_render_fused_forward(B, W, H, K, float(focallength), ptr(indices), ptr(points), ptr(normals),
                                     stdDevs.shape[0], N, ptr(stdDevs), float(smoothing), attribute.shape[0], C,
                                     ptr(attribute), ptr(weights), ptr(depth), ptr(image), ptr(ws), ws.numel(),
                                     stream_ptr(points.device)), "render forward")
    return image, depth, weights


def renderBackward(width: int, height: int, focallength: float, gradImage, gradDepthWeights, gradWeights, indices,
                   weights, points, normals, stdDevs, smoothing: float, attribute):
    """Backward of renderForward: gradients of the image (and, if not None,
    of the depth weights and the EWA weights) -> [grad points, grad normals,
    grad std-devs (the EWA kernel's raw gradients), grad attribute]."""
    _check(indices, points, normals, stdDevs)
    dev = points.device
    need(gradImage, "gradImage", device=dev)
    need(weights, "weights", device=dev)
    need(attribute, "attribute", device=dev)
    for name, g in (("gradDepthWeights", gradDepthWeights), ("gradWeights", gradWeights)):
        if g is not None:
            need(g, name, device=dev)
            if g.shape != indices.shape:
                raise ValueError(f"{name} must match indices")
    B, W, H, K = indices.shape
    N, C = points.shape[1], attribute.shape[2]
    if tuple(gradImage.shape) != (B, W, H, C) or weights.shape != indices.shape:
        raise ValueError("gradImage must be (B,W,H,C) and weights (B,W,H,K)")
    L = load()
    ws = Workspace.get(dev, L.uds_splat_workspace_size(B, N), "splat")
    gp, gn, gs, ga = (torch.empty_like(t) for t in (points, normals, stdDevs, attribute))
    check(L.uds_render_fused_backward(B, W, H, K, float(focallength), ptr(gradImage), ptr(gradDepthWeights),
                                      ptr(gradWeights), ptr(indices), ptr(weights), ptr(points), ptr(normals),
                                      stdDevs.shape[0], N, ptr(stdDevs), float(smoothing), attribute.shape[0], C,
                                      ptr(attribute), ptr(gp), ptr(gn), ptr(gs), ptr(ga), ptr(ws), ws.numel(),
                                      stream_ptr(dev)), "render backward")
    return [gp, gn, gs, ga]
