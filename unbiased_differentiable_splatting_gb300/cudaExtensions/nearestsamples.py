"""cudaExtensions.nearestsamples (nearestSamples.cpp:31-75).

``nearest(indices (B,W,H,K) int32, weights (B,W,H,K), points (1,N,3),
numNearest)`` -> (1,N,numNearest) int32: for every splat, its nearest other
splats among the samples of the pixels where it is the surface sample
(largest weight), ordered by (distance, index) and padded with -1.

``regularizer(nearest, points, normals, sigma, mean)`` -> (losses (2,),
grad_points (N,3), grad_normals (N,3)): the normal and plane losses of the
nearest-sample regulariser (regularizier.py:119-175) and their gradients
w.r.t. each splat's own point and normal, in one kernel (no counterpart
module in the reference; its regulariser composes these from tensor ops).
"""
from __future__ import annotations

import torch

from .._lib import Workspace, check, load, need, ptr, stream_ptr


def nearest(indices, weights, points, numNearest):
    need(indices, "indices", torch.int32)
    need(weights, "weights", device=indices.device)
    need(points, "points", device=indices.device)
    B, W, H, K = indices.shape
    if tuple(weights.shape) != (B, W, H, K):
        raise ValueError("weights must match indices")
    if points.dim() != 3 or points.shape[0] != 1 or points.shape[2] != 3:
        raise ValueError("points must be (1,N,3)")
    N, M = points.shape[1], int(numNearest)
    out = torch.empty((1, N, M), dtype=torch.int32, device=indices.device)
    L = load()
    ws = Workspace.get(indices.device, L.uds_nearest_workspace_size(B, W, H, K, N), "nearest")
    check(L.uds_nearest_samples(B, W, H, K, ptr(indices), ptr(weights), N, ptr(points), M, ptr(out), ptr(ws),
                                ws.numel(), stream_ptr(indices.device)), "nearestsamples nearest")
    return out


def regularizer(nearest, points, normals, sigma, mean=False):
    need(nearest, "nearest", torch.int32)
    need(points, "points", device=nearest.device)
    need(normals, "normals", device=nearest.device)
    if nearest.dim() != 3 or nearest.shape[0] != 1 or points.dim() != 3 or points.shape[0] != 1 or \
            points.shape[2] != 3 or normals.shape != points.shape or nearest.shape[1] != points.shape[1]:
        raise ValueError("nearest must be (1,N,M) and points / normals (1,N,3)")
    N, M = points.shape[1], nearest.shape[2]
    dev = points.device
    losses = torch.empty(2, dtype=torch.float32, device=dev)
    gp = torch.empty((1, N, 3), dtype=torch.float32, device=dev)
    gn = torch.empty((1, N, 3), dtype=torch.float32, device=dev)
    L = load()
    ws = Workspace.get(dev, L.uds_nearest_regularizer_workspace_size(N), "regularizer")
    check(L.uds_nearest_regularizer(N, M, ptr(nearest), ptr(points), ptr(normals), float(sigma), int(bool(mean)),
                                    ptr(losses), ptr(gp), ptr(gn), ptr(ws), ws.numel(), stream_ptr(dev)),
          "nearestsamples regularizer")
    return losses, gp, gn
