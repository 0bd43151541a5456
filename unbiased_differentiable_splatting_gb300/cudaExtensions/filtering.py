"""cudaExtensions.filtering (zSorting.cpp:24-43): per-pixel depth ordering and
front-to-back alpha blending of the EWA weights."""
from __future__ import annotations

import torch

from .._lib import check, load, need, ptr, stream_ptr


def _check(indices, weights, points, normals):
    need(indices, "indices", torch.int32)
    dev = indices.device
    need(weights, "weights", device=dev)
    need(points, "points", device=dev)
    need(normals, "normals", device=dev)
    if indices.shape != weights.shape or indices.dim() != 4:
        raise ValueError("indices and weights must both be (B,W,H,K)")
    if points.shape != normals.shape or points.shape[0] not in (1, indices.shape[0]):
        raise ValueError("points/normals must be (1|B,N,3)")


def forward(indices, weights, width: int, height: int, focallength: float, points, normals):
    _check(indices, weights, points, normals)
    B, W, H, K = indices.shape
    out = torch.empty_like(weights)
    check(load().uds_filter_forward(B, W, H, K, ptr(indices), ptr(weights), float(focallength), points.shape[0],
                                    points.shape[1], ptr(points), ptr(normals), ptr(out), stream_ptr(points.device)),
          "filtering forward")
    return out


def backward(indices, weights, gradIn, width: int, height: int, focallength: float, points, normals):
    _check(indices, weights, points, normals)
    need(gradIn, "gradIn", device=indices.device)
    B, W, H, K = indices.shape
    out = torch.empty_like(weights)
    check(load().uds_filter_backward(B, W, H, K, ptr(indices), ptr(weights), ptr(gradIn), float(focallength),
                                     points.shape[0], points.shape[1], ptr(points), ptr(normals), ptr(out),
                                     stream_ptr(points.device)), "filtering backward")
    return out
