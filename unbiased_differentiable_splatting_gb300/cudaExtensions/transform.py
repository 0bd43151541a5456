"""cudaExtensions.transform (transform.cpp:33-86), and the view matrix of
world2Camera (utils.py:11-49)."""
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


def viewMatrixForward(positions: torch.Tensor, quaternions: torch.Tensor) -> torch.Tensor:
    """(B, 3) positions, (B, 4) quaternions (x, y, z, w) -> (B, 1, 4, 4)."""
    need(positions, "positions")
    need(quaternions, "quaternions", device=positions.device)
    B = quaternions.shape[0]
    out = torch.empty((B, 1, 4, 4), dtype=torch.float32, device=positions.device)
    check(load().uds_view_matrix_forward(B, ptr(positions), ptr(quaternions), ptr(out), stream_ptr(positions.device)),
          "view matrix forward")
    return out


def viewMatrixBackward(gradIn: torch.Tensor, quaternions: torch.Tensor):
    need(gradIn, "gradIn")
    need(quaternions, "quaternions", device=gradIn.device)
    B = quaternions.shape[0]
    gp = torch.empty((B, 3), dtype=torch.float32, device=gradIn.device)
    gq = torch.empty_like(quaternions)
    check(load().uds_view_matrix_backward(B, ptr(gradIn), ptr(quaternions), ptr(gp), ptr(gq),
                                          stream_ptr(gradIn.device)), "view matrix backward")
    return gp, gq
