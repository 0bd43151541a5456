"""cudaExtensions.pixelgather (pixelGather.cpp:10-24, pixelGatherCuda.cu:7-152).

``scatter(indices (B,W,H,K) int32, values (B,N,C))`` -> (B,W,H,K,C): each
sample's splat attributes (0 where the index is -1).
``gather(indices, values (B,W,H,K,C), numSources)`` -> (B,N,C): per-splat sum
of the samples' values (the backward of scatter, and the visibility count of
cleanup.py:41).  ``deterministic=True`` (an addition) sums each splat's
samples in sample order instead of with atomics, so repeated calls give
identical bits.
"""
from __future__ import annotations

import torch

from .._lib import Workspace, check, load, need, ptr, stream_ptr


def scatter(indices, values):
    need(indices, "indices", torch.int32)
    need(values, "values", device=indices.device)
    B, W, H, K = indices.shape
    if values.dim() != 3 or values.shape[0] != B:
        raise ValueError("values must be (B,N,C) with the indices' B")
    N, C = values.shape[1], values.shape[2]
    out = torch.empty((B, W, H, K, C), device=indices.device)
    check(load().uds_pixel_scatter(B, W, H, K, ptr(indices), N, C, ptr(values), ptr(out),
                                   stream_ptr(indices.device)), "pixelgather scatter")
    return out


def gather(indices, values, numSources, deterministic=False):
    need(indices, "indices", torch.int32)
    need(values, "values", device=indices.device)
    B, W, H, K = indices.shape
    if values.dim() != 5 or tuple(values.shape[:4]) != (B, W, H, K):
        raise ValueError("values must be (B,W,H,K,C)")
    N, C = int(numSources), values.shape[4]
    out = torch.empty((B, N, C), device=indices.device)
    L = load()
    ws = None
    if deterministic:
        ws = Workspace.get(indices.device, L.uds_pixel_gather_workspace_size(B, W, H, K, N), "pixelgather")
    check(L.uds_pixel_gather(B, W, H, K, ptr(indices), N, C, ptr(values), ptr(out), int(bool(deterministic)),
                             ptr(ws), ws.numel() if ws is not None else 0, stream_ptr(indices.device)),
          "pixelgather gather")
    return out
