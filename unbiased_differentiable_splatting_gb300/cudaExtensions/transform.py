"""cudaExtensions.transform (transform.cpp:33-86)."""
from __future__ import annotations

import torch

from .._lib import check, load, need, ptr, stream_ptr


def _forward(affine: bool, transformation: torch.Tensor, vector: torch.Tensor) -> torch.Tensor:
    need(transformation, "transformation")
    need(vector, "vector", device=transformation.device)
    B, N = transformation.shape[0], vector.shape[1]
    if transformation.shape[1:] != (4, 4) or vector.dim() != 3 or vector.shape[2] != 3:
        raise ValueError("expected transformation (B,4,4) and vector (1|B,N,3)")
    out = torch.empty((B, N, 3), dtype=vector.dtype, device=vector.device)
    check(load().uds_transform_forward(int(affine), B, ptr(transformation), vector.shape[0], N, ptr(vector),
                                       ptr(out), stream_ptr(vector.device)), "transform forward")
    return out


def _backward(affine: bool, gradIn: torch.Tensor, transformation: torch.Tensor, vector: torch.Tensor):
    need(gradIn, "gradIn")
    need(transformation, "transformation", device=gradIn.device)
    need(vector, "vector", device=gradIn.device)
    B, N = transformation.shape[0], vector.shape[1]
    if tuple(gradIn.shape) != (B, N, 3):
        raise ValueError("gradIn must have shape (B,N,3)")
    gM = torch.empty_like(transformation)
    gv = torch.empty_like(vector)
    check(load().uds_transform_backward(int(affine), B, ptr(gradIn), ptr(transformation), vector.shape[0], N,
                                        ptr(vector), ptr(gM), ptr(gv), stream_ptr(vector.device)),
          "transform backward")
    return [gM, gv]


def affineForward(transformation, vector):
    return _forward(True, transformation, vector)


def affineBackward(gradIn, transformation, vector):
    return _backward(True, gradIn, transformation, vector)


def linearForward(transformation, vector):
    return _forward(False, transformation, vector)


def linearBackward(gradIn, transformation, vector):
    return _backward(False, gradIn, transformation, vector)
