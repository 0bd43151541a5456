"""cudaExtensions.interpolation (interpolation.cpp:31-95)."""
from __future__ import annotations

import torch

from .._lib import check, load, need, ptr, stream_ptr


def _check(indices, weights, attribute):
    need(indices, "indices", torch.int32)
    need(weights, "weights", device=indices.device)
    need(attribute, "attribute", device=indices.device)
    if indices.shape != weights.shape or indices.dim() != 4 or attribute.dim() != 3:
        raise ValueError("expected indices/weights (B,W,H,K) and attribute (1|B,N,C)")
    if attribute.shape[0] not in (1, indices.shape[0]):
        raise ValueError("attribute batch must be 1 or B")


def forward(indices, weights, attribute):
    _check(indices, weights, attribute)
    B, W, H, K = indices.shape
    C = attribute.shape[2]
    out = torch.empty((B, W, H, C), dtype=torch.float32, device=indices.device)
    check(load().uds_interp_forward(B, W, H, K, ptr(indices), ptr(weights), attribute.shape[0], attribute.shape[1],
                                    C, ptr(attribute), ptr(out), stream_ptr(indices.device)), "interpolation forward")
    return out


def backward(gradIn, indices, weights, attribute):
    _check(indices, weights, attribute)
    need(gradIn, "gradIn", device=indices.device)
    B, W, H, K = indices.shape
    C = attribute.shape[2]
    gw = torch.empty_like(weights)
    ga = torch.empty_like(attribute)
    check(load().uds_interp_backward(B, W, H, K, ptr(gradIn), ptr(indices), ptr(weights), attribute.shape[0],
                                     attribute.shape[1], C, ptr(attribute), ptr(gw), ptr(ga),
                                     stream_ptr(indices.device)), "interpolation backward")
    return [gw, ga]
