"""cudaExtensions.transform (transform.cpp:33-86), the view matrix of
world2Camera (utils.py:11-49) and the normal flips of BackfaceCulling
(render.py:193-205)."""
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


def backfaceForward(camNormals: torch.Tensor, normals=None):
    """(B,N,3) camera-space normals, optional (1|B,N,3) world normals ->
    [flipped camera-space normals (B,N,3)] + [flipped world normals (B,N,3)]
    when normals is given."""
    need(camNormals, "camNormals")
    if camNormals.dim() != 3 or camNormals.shape[2] != 3:
        raise ValueError("camNormals must be (B,N,3)")
    B, N = camNormals.shape[0], camNormals.shape[1]
    fc = torch.empty_like(camNormals)
    fw = None
    if normals is not None:
        need(normals, "normals", device=camNormals.device)
        if normals.dim() != 3 or normals.shape[1:] != camNormals.shape[1:] or normals.shape[0] not in (1, B):
            raise ValueError("normals must be (1|B,N,3)")
        fw = torch.empty_like(camNormals)
    check(load().uds_backface_forward(B, N, ptr(camNormals), normals.shape[0] if normals is not None else 1,
                                      ptr(normals), ptr(fc), ptr(fw), stream_ptr(camNormals.device)),
          "backface forward")
    return [fc] if fw is None else [fc, fw]


def backfaceBackward(camNormals: torch.Tensor, gradCam=None, gradNormals=None, normalsBatch: int = 1):
    """Gradients of backfaceForward: [grad camNormals or None, grad normals
    (normalsBatch,N,3) or None]."""
    need(camNormals, "camNormals")
    B, N = camNormals.shape[0], camNormals.shape[1]
    gc = gw = None
    if gradCam is not None:
        need(gradCam, "gradCam", device=camNormals.device)
        gc = torch.empty_like(camNormals)
    if gradNormals is not None:
        need(gradNormals, "gradNormals", device=camNormals.device)
        gw = torch.empty((normalsBatch, N, 3), dtype=torch.float32, device=camNormals.device)
    check(load().uds_backface_backward(B, N, ptr(camNormals), ptr(gradCam), normalsBatch, ptr(gradNormals), ptr(gc),
                                       ptr(gw), stream_ptr(camNormals.device)), "backface backward")
    return gc, gw
