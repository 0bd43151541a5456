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
