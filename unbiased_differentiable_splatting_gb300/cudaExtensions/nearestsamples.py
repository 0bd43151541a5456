"""cudaExtensions.nearestsamples (nearestSamples.cpp:31-75).

``nearest(indices (B,W,H,K) int32, weights (B,W,H,K), points (1,N,3),
numNearest)`` -> (1,N,numNearest) int32: for every splat, its nearest other
splats among the samples of the pixels where it is the surface sample
(largest weight), ordered by (distance, index) and padded with -1.
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
