"""Autograd wrappers over the CUDA ops, with the class names, call signatures
and gradient conventions of the reference's ``splatting/extensions/__init__.py``
(lines 104-581) and the helpers of ``splatting/extensions/utils.py``.

Every class calls the ops registered in ``library`` (``torch.ops.uds.*``), so
the dispatcher, fake tensors and ``torch.compile`` see them.

Gradient conventions kept from the reference:
* ``EWASplatting.backward`` clamps each splat's point / std-dev gradient to
  norm <= 1 (``conditionalNormalization``), zeroes NaNs and returns no gradient
  for the normals (extensions/__init__.py:219-233);
* ``DepthFiltering`` passes gradients only to the EWA weights;
* the sampler runs under ``no_grad``.
"""
from __future__ import annotations

import torch as th

from . import library  # noqa: F401  (registers torch.ops.uds)
from .cudaExtensions import sampling

ops = th.ops.uds


# ------------------------------------------------------------------ utils
def normalize(x: th.Tensor, eps=1e-4) -> th.Tensor:
    """utils.py:7-9"""
    norm = x.norm(dim=-1, keepdim=True)
    return x / (norm + eps)


def dot(x: th.Tensor, y: th.Tensor, keepdim: bool) -> th.Tensor:
    return th.sum(x.mul(y), dim=-1, keepdim=keepdim)


class ViewMatrix(th.autograd.Function):
    """world2Camera on the GPU: one kernel each way (the forward rounds like
    the reference's tensor operations, so the matrix is the same)."""

    @staticmethod
    def forward(ctx, camPositions, camQuaternion):
        q = camQuaternion.contiguous()
        ctx.save_for_backward(q)
        ctx.pshape = camPositions.shape
        return ops.view_matrix_forward(camPositions.reshape(-1, 3).contiguous(), q)

    @staticmethod
    def backward(ctx, gradIn):
        (q,) = ctx.saved_tensors
        gp, gq = ops.view_matrix_backward(gradIn.contiguous(), q)
        return gp.reshape(ctx.pshape), gq


def world2Camera(camPositions: th.Tensor, camQuaternion: th.Tensor) -> th.Tensor:
    """Quaternion (x, y, z, w) + translation -> (B,1,4,4) view matrix
    (Euler-Rodrigues rotation, utils.py:11-49): the fused kernels for float32
    CUDA tensors of shapes (B,3) and (B,4), else the tensor expression."""
    B = camPositions.shape[0]
    if (camPositions.is_cuda and camQuaternion.is_cuda and camPositions.dtype == th.float32
            and camQuaternion.dtype == th.float32 and camPositions.device == camQuaternion.device
            and camQuaternion.dim() == 2 and camQuaternion.shape[1] == 4 and camPositions.numel() == 3 * B
            and camQuaternion.shape[0] == B):
        return ViewMatrix.apply(camPositions, camQuaternion)
    x, y, z, w = camQuaternion.split(1, dim=-1)
    x2, y2, z2, w2 = x * x, y * y, z * z, w * w
    xy, zw, xz, yw, yz, xw = x * y, z * w, x * z, y * w, y * z, x * w
    row0 = th.cat([x2 - y2 - z2 + w2, 2 * (xy - zw), 2 * (xz + yw)], dim=-1)
    row1 = th.cat([2 * (xy + zw), -x2 + y2 - z2 + w2, 2 * (yz - xw)], dim=-1)
    row2 = th.cat([2 * (xz - yw), 2 * (yz + xw), -x2 - y2 + z2 + w2], dim=-1)
    R = th.stack([row0, row1, row2], dim=-2)  # (B,3,3)
    top = th.cat([R, camPositions.reshape(B, 3, 1)], dim=-1)
    bottom = th.zeros((B, 1, 4), dtype=camPositions.dtype, device=camPositions.device)
    bottom[..., 3] = 1.0
    return th.cat([top, bottom], dim=-2).unsqueeze(1)


def transformForward(viewMatrix: th.Tensor, forward: str) -> th.Tensor:
    """utils.py:51-60: for forward == 'z' flip y and mirror z."""
    if forward == "z":
        d = th.ones(4, dtype=viewMatrix.dtype, device=viewMatrix.device)
        d[1:3] = -1.0  # built on the device: no host copy, so CUDA-graph capture works
        flip = th.diag(d)
        viewMatrix = flip.view(1, 1, 4, 4) @ viewMatrix
    return viewMatrix


def conditionalNormalization(dx: th.Tensor, radius=1.0, eps=1e-4) -> th.Tensor:
    """utils.py:147-150: scale rows with norm > 1 down to norm ~1."""
    norm = dx.norm(dim=-1, keepdim=True)
    scale = th.clamp(norm + eps, 1.0)
    return dx.div(scale)


# --------------------------------------------------------------- sampling
class FmmSampling:
    """extensions/__init__.py:106-117.  Calls ``torch.ops.uds.sample`` when the
    keyword arguments are at most ``seed`` and ``uniforms``; the additions the
    op schema leaves out (``h``, ``return_stats``, ``tile_x``, ...) go to
    ``cudaExtensions.sampling.sample`` directly."""

    @th.no_grad()
    def __call__(self, width: int, height: int, focallength: float, points: th.Tensor, normals: th.Tensor,
                 colors: th.Tensor, stdDevs: th.Tensor, numSamples: int, smoothing: float,
                 precision: float = 0.001, **kwargs) -> th.Tensor:
        if set(kwargs) <= {"seed", "uniforms"}:
            seed = kwargs.get("seed")
            if seed is None:
                seed = int(th.randint(0, 2 ** 62, (1,)).item())
            tensor_seed = isinstance(seed, th.Tensor)
            if not tensor_seed:  # the 64-bit Philox key as the schema's signed int64
                seed = int(seed) & 0xFFFFFFFFFFFFFFFF
                seed = seed - (1 << 64) if seed >= (1 << 63) else seed
            return ops.sample(int(width), int(height), float(focallength), points, normals, stdDevs, int(numSamples),
                              float(smoothing), float(precision), 0 if tensor_seed else int(seed),
                              seed if tensor_seed else None, kwargs.get("uniforms"))
        return sampling.sample(width, height, focallength, points, normals, colors, stdDevs, numSamples, smoothing,
                               precision, **kwargs)


# --------------------------------------------------------------- transform
class AffineTransform(th.autograd.Function):
    @staticmethod
    def forward(ctx, transformMatrix, vector):
        ctx.save_for_backward(transformMatrix, vector)
        return ops.affine_forward(transformMatrix.contiguous(), vector.contiguous())

    @staticmethod
    def backward(ctx, gradIn):
        M, v = ctx.saved_tensors
        gM, gv = ops.affine_backward(gradIn.contiguous(), M.contiguous(), v.contiguous())
        return gM, gv


class LinearTransform(th.autograd.Function):
    @staticmethod
    def forward(ctx, transformMatrix, vector):
        ctx.save_for_backward(transformMatrix, vector)
        return ops.linear_forward(transformMatrix.contiguous(), vector.contiguous())

    @staticmethod
    def backward(ctx, gradIn):
        M, v = ctx.saved_tensors
        gM, gv = ops.linear_backward(gradIn.contiguous(), M.contiguous(), v.contiguous())
        return gM, gv


# ------------------------------------------------------------------- EWA
class EWASplatting(th.autograd.Function):
    @staticmethod
    def forward(ctx, width: int, height: int, focallength: float, indices: th.Tensor, points: th.Tensor,
                normals: th.Tensor, stdDevs: th.Tensor, smoothing: float) -> th.Tensor:
        points, normals, stdDevs = points.contiguous(), normals.contiguous(), stdDevs.contiguous()
        weights = ops.splat_forward(width, height, float(focallength), indices, points, normals, stdDevs,
                                    float(smoothing))
        ctx.save_for_backward(indices, points, normals, stdDevs)
        ctx.width, ctx.height, ctx.focallength, ctx.smoothing = width, height, focallength, smoothing
        return weights

    @staticmethod
    def backward(ctx, gradWeights):
        indices, points, normals, stdDevs = ctx.saved_tensors
        gradPoints, gradNormals, gradStdDevs = ops.splat_backward(ctx.width, ctx.height, float(ctx.focallength),
                                                                  gradWeights.contiguous(), indices, points, normals,
                                                                  stdDevs, float(ctx.smoothing))
        gradPoints = conditionalNormalization(gradPoints)
        gradStdDevs = conditionalNormalization(gradStdDevs)
        gradPoints = th.nan_to_num(gradPoints, nan=0.0, posinf=float("inf"), neginf=float("-inf"))
        gradStdDevs = th.nan_to_num(gradStdDevs, nan=0.0, posinf=float("inf"), neginf=float("-inf"))
        return None, None, None, None, gradPoints, None, gradStdDevs, None


# ------------------------------------------------------------ compositing
class DepthFiltering(th.autograd.Function):
    @staticmethod
    def forward(ctx, indices, weights, width: int, height: int, focallength: float, points, normals):
        weights, points, normals = weights.contiguous(), points.contiguous(), normals.contiguous()
        ctx.save_for_backward(indices, weights, points, normals)
        ctx.width, ctx.height, ctx.focallength = width, height, focallength
        return ops.filter_forward(indices, weights, width, height, float(focallength), points, normals)

    @staticmethod
    def backward(ctx, gradIn):
        indices, weights, points, normals = ctx.saved_tensors
        gradWeights = ops.filter_backward(indices, weights, gradIn.contiguous(), ctx.width, ctx.height,
                                          float(ctx.focallength), points, normals)
        return None, gradWeights, None, None, None, None, None


# ---------------------------------------------------------- interpolation
class LinearInterpolation(th.autograd.Function):
    @staticmethod
    def forward(ctx, indices, weights, values):
        weights, values = weights.contiguous(), values.contiguous()
        ctx.save_for_backward(indices, weights, values)
        return ops.interp_forward(indices, weights, values)

    @staticmethod
    def backward(ctx, gradIn):
        indices, weights, values = ctx.saved_tensors
        gradWeights, gradValues = ops.interp_backward(gradIn.contiguous(), indices, weights, values)
        return None, gradWeights, gradValues


# ---------------------------------------------------------------- shading
class DiffuseShading(th.autograd.Function):
    @staticmethod
    def forward(ctx, directions, intensites, normals, diffuse):
        directions, intensites = directions.contiguous(), intensites.contiguous()
        normals, diffuse = normals.contiguous(), diffuse.contiguous()
        ctx.save_for_backward(directions, intensites, normals, diffuse)
        return ops.shade_forward(directions, intensites, normals, diffuse)

    @staticmethod
    def backward(ctx, gradIn):
        directions, intensites, normals, diffuse = ctx.saved_tensors
        return tuple(ops.shade_backward(gradIn.contiguous(), directions, intensites, normals, diffuse))


class LambertShading(th.autograd.Function):
    """Per-splat Lambert of the forward shading mode (shading.py:12-29),
    fused into one kernel each way."""

    @staticmethod
    def forward(ctx, ambient, directions, intensities, normals, diffuse):
        ts = [t.contiguous() for t in (ambient, directions, intensities, normals, diffuse)]
        ctx.save_for_backward(*ts)
        return ops.lambert_forward(*ts)

    @staticmethod
    def backward(ctx, gradIn):
        return tuple(ops.lambert_backward(gradIn.contiguous(), *ctx.saved_tensors))


class SphericalHarmonicShading(th.autograd.Function):
    @staticmethod
    def forward(ctx, coefficients, normals, diffuse):
        coefficients, normals, diffuse = coefficients.contiguous(), normals.contiguous(), diffuse.contiguous()
        ctx.save_for_backward(coefficients, normals, diffuse)
        return ops.shade_sh_forward(coefficients, normals, diffuse)

    @staticmethod
    def backward(ctx, gradIn):
        coefficients, normals, diffuse = ctx.saved_tensors
        return tuple(ops.shade_sh_backward(gradIn.contiguous(), coefficients, normals, diffuse))


__all__ = ["FmmSampling", "AffineTransform", "LinearTransform", "EWASplatting", "DepthFiltering",
           "LinearInterpolation", "DiffuseShading", "LambertShading", "SphericalHarmonicShading", "world2Camera",
           "transformForward",
           "conditionalNormalization", "normalize", "dot"]


# ------------------------------------------------------------ pixel gather
class PixelScatterGather(th.autograd.Function):
    """extensions/__init__.py:407-437: per-sample splat attributes
    (B,W,H,K,C) from (B,N,C); the backward sums each sample's gradient back
    onto its splat."""

    @staticmethod
    def forward(ctx, indices, values):
        ctx.save_for_backward(indices)
        ctx.numSources = values.shape[1]
        return ops.pixel_scatter(indices, values.contiguous())

    @staticmethod
    def backward(ctx, grad_output):
        (indices,) = ctx.saved_tensors
        return None, ops.pixel_gather(indices, grad_output.contiguous(), ctx.numSources, False)
