"""Autograd wrappers over the CUDA ops, with the class names, call signatures
and gradient conventions of the reference's ``splatting/extensions/__init__.py``
(lines 104-581) and the helpers of ``splatting/extensions/utils.py``.

Every class is a thin callable over the ops registered in ``library``
(``torch.ops.uds.*``, whose autograd formulas are registered with the
dispatcher), so fake tensors and ``torch.compile`` see them; ``X.apply(...)``
takes the reference's arguments.

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


def world2Camera(camPositions: th.Tensor, camQuaternion: th.Tensor) -> th.Tensor:
    """Quaternion (x, y, z, w) + translation -> (B,1,4,4) view matrix
    (Euler-Rodrigues rotation, utils.py:11-49): the fused kernels for float32
    CUDA tensors of shapes (B,3) and (B,4), else the tensor expression."""
    B = camPositions.shape[0]
    if (camPositions.is_cuda and camQuaternion.is_cuda and camPositions.dtype == th.float32
            and camQuaternion.dtype == th.float32 and camPositions.device == camQuaternion.device
            and camQuaternion.dim() == 2 and camQuaternion.shape[1] == 4 and camPositions.numel() == 3 * B
            and camQuaternion.shape[0] == B):
        return ops.view_matrix_forward(camPositions.reshape(B, 3).contiguous(), camQuaternion.contiguous())
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
    keyword arguments are at most ``seed``, ``uniforms`` and ``leaf_size``;
    the additions the op schema leaves out (``h``, ``return_stats``,
    ``tile_x``, ...) go to ``cudaExtensions.sampling.sample`` directly."""

    @th.no_grad()
    def __call__(self, width: int, height: int, focallength: float, points: th.Tensor, normals: th.Tensor,
                 colors: th.Tensor, stdDevs: th.Tensor, numSamples: int, smoothing: float,
                 precision: float = 0.001, **kwargs) -> th.Tensor:
        if set(kwargs) <= {"seed", "uniforms", "leaf_size"}:
            seed = kwargs.get("seed")
            if seed is None:
                seed = int(th.randint(0, 2 ** 62, (1,)).item())
            tensor_seed = isinstance(seed, th.Tensor)
            if not tensor_seed:  # the 64-bit Philox key as the schema's signed int64
                seed = int(seed) & 0xFFFFFFFFFFFFFFFF
                seed = seed - (1 << 64) if seed >= (1 << 63) else seed
            return ops.sample(int(width), int(height), float(focallength), points, normals, stdDevs, int(numSamples),
                              float(smoothing), float(precision), 0 if tensor_seed else int(seed),
                              seed if tensor_seed else None, kwargs.get("uniforms"),
                              int(kwargs.get("leaf_size") or 0))
        return sampling.sample(width, height, focallength, points, normals, colors, stdDevs, numSamples, smoothing,
                               precision, **kwargs)


class _OpFunction:
    """A reference autograd-Function name over a registered op: ``apply``
    takes the reference's arguments, makes the tensors contiguous and calls
    the op, whose autograd formula is registered with the dispatcher (so
    torch.compile traces it without an autograd.Function)."""

    op_name = ""

    @classmethod
    def apply(cls, *args):
        args = [a.contiguous() if isinstance(a, th.Tensor) else a for a in args]
        return getattr(ops, cls.op_name)(*args)


# --------------------------------------------------------------- transform
class AffineTransform(_OpFunction):
    """AffineTransform.apply(M (B,4,4), v (1|B,N,3)) -> (B,N,3)."""
    op_name = "affine_forward"


class LinearTransform(_OpFunction):
    """LinearTransform.apply(M (B,4,4), v (1|B,N,3)) -> (B,N,3)."""
    op_name = "linear_forward"


# ------------------------------------------------------------------- EWA
class EWASplatting(_OpFunction):
    """EWASplatting.apply(width, height, focallength, indices, points,
    normals, stdDevs, smoothing) -> weights (B,W,H,K); gradients with the
    reference's post-processing (``torch.ops.uds.ewa_weights``)."""

    @classmethod
    def apply(cls, width, height, focallength, indices, points, normals, stdDevs, smoothing):
        return ops.ewa_weights(int(width), int(height), float(focallength), indices, points.contiguous(),
                               normals.contiguous(), stdDevs.contiguous(), float(smoothing))


# ------------------------------------------------------------ compositing
class DepthFiltering(_OpFunction):
    """DepthFiltering.apply(indices, weights, width, height, focallength,
    points, normals) -> depth weights; gradients for the weights only."""

    @classmethod
    def apply(cls, indices, weights, width, height, focallength, points, normals):
        return ops.filter_forward(indices, weights.contiguous(), int(width), int(height), float(focallength),
                                  points.contiguous(), normals.contiguous())


# ---------------------------------------------------------- interpolation
class LinearInterpolation(_OpFunction):
    """LinearInterpolation.apply(indices, weights, values (1|B,N,C))."""
    op_name = "interp_forward"


# ---------------------------------------------------------------- shading
class DiffuseShading(_OpFunction):
    """DiffuseShading.apply(directions, intensities, normals, diffuse)."""
    op_name = "shade_forward"


class LambertShading(_OpFunction):
    """Per-splat Lambert of the forward shading mode (shading.py:12-29),
    one kernel each way: apply(ambient, directions, intensities, normals,
    diffuse)."""
    op_name = "lambert_forward"


class SphericalHarmonicShading(_OpFunction):
    """SphericalHarmonicShading.apply(coefficients, normals, diffuse)."""
    op_name = "shade_sh_forward"


__all__ = ["FmmSampling", "AffineTransform", "LinearTransform", "EWASplatting", "DepthFiltering",
           "LinearInterpolation", "DiffuseShading", "LambertShading", "SphericalHarmonicShading", "world2Camera",
           "transformForward",
           "conditionalNormalization", "normalize", "dot"]


# ------------------------------------------------------------ pixel gather
class PixelScatterGather(_OpFunction):
    """extensions/__init__.py:407-437: per-sample splat attributes
    (B,W,H,K,C) from (B,N,C); the backward sums each sample's gradient back
    onto its splat (apply(indices, values))."""
    op_name = "pixel_scatter"
