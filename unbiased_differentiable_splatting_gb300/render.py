"""Renderer module with the interface of the reference's ``splatting/render.py``
(``Splatting``, render.py:230-376) and the per-splat shading modules of
``splatting/shading.py``.

``Splatting.forward`` runs: world->camera transform of points and normals,
back-face orientation, FMM sampling of K splats per pixel, EWA weights, depth
compositing, shading / attribute interpolation.  Every stage is a CUDA op of
libuds.so behind the autograd wrappers of ``extensions``; for the shading
modes that interpolate one per-splat attribute (forward, forwardHarmonics,
None) the EWA weights, compositing and interpolation run as one fused kernel
each way (``torch.ops.uds.render_splats``), with the same results.

Difference from the reference: ``self.indices`` (render.py:296 copies the
indices to the host on every forward) is a lazy property here, so a forward
pass never synchronises with the host.
"""
from __future__ import annotations

import math
from dataclasses import dataclass

import torch as th

from .cudaExtensions import shading as _shading
from .extensions import (AffineTransform, DepthFiltering, DiffuseShading, EWASplatting, FmmSampling,
                         LambertShading, LinearInterpolation, LinearTransform, SphericalHarmonicShading, dot,
                         normalize, transformForward, world2Camera)


@dataclass
class RenderOptions:
    """The argparse fields Splatting reads (optimization_geometry.py:60-121)."""

    forward: str = "-z"
    numSamples: int = 40
    precision: float = 0.01
    shadingMode: str = "forward"
    dtype: str = "float"
    device: str = "cuda:0"


def _cosine(normal: th.Tensor, light: th.Tensor) -> th.Tensor:
    return th.clamp(th.sum(light.mul(normal), dim=-1, keepdim=True), 0.0, 1.0)


class BackfaceCulling(th.nn.Module):
    """render.py:193-205: flip normals that face away from the camera, in one
    kernel (``torch.ops.uds.backface``, differentiable).  With ``normals``
    None only the camera-space normals are flipped (the shading modes that do
    not read the flipped world normals)."""

    def forward(self, normals, camNormals):
        out = th.ops.uds.backface(camNormals.contiguous(), None if normals is None else normals.contiguous())
        return (None if normals is None else out[1]), out[0]


class Lambert(th.nn.Module):
    """shading.py:12-29: per-splat ambient + Lambert shading: one fused kernel
    each way when the operands have the shapes it takes (the renderer's),
    else the reference's tensor expression."""

    def forward(self, ambientLight, lampDirections, lampIntensities, normals, diffuse):
        if _shading.lambert_shapes(ambientLight, lampDirections, lampIntensities, normals, diffuse) is not None:
            return LambertShading.apply(ambientLight, lampDirections, lampIntensities, normals, diffuse)
        bn, l, _ = lampDirections.shape
        lampDirections = lampDirections.view(bn, l, 1, 3)
        normals = normals.unsqueeze(1)
        ambientIrradiance = ambientLight * diffuse
        radiance = lampIntensities.view(lampIntensities.shape[0], l, 1, 3)
        irradiance = radiance.mul(_cosine(normals, lampDirections))
        brdf = diffuse.unsqueeze(1) / math.pi
        return ambientIrradiance + th.mul(irradiance, brdf).sum(dim=1)


def _sh_matrix(coefficients: th.Tensor) -> th.Tensor:
    c1, c2, c3, c4, c5 = 0.429043, 0.511664, 0.743125, 0.886227, 0.247708
    c = coefficients
    M = th.stack([
        th.stack([c1 * c[..., 8], c1 * c[..., 4], c1 * c[..., 7], c2 * c[..., 3]], -1),
        th.stack([c1 * c[..., 4], -c1 * c[..., 8], c1 * c[..., 5], c2 * c[..., 1]], -1),
        th.stack([c1 * c[..., 7], c1 * c[..., 5], c3 * c[..., 6], c2 * c[..., 2]], -1),
        th.stack([c2 * c[..., 3], c2 * c[..., 1], c2 * c[..., 2], c4 * c[..., 0] - c5 * c[..., 6]], -1),
    ], -1)
    return M  # symmetric; column j is the j-th stacked vector


class ForwardSphericalHaromic(th.nn.Module):
    """shading.py:79-129: per-splat order-2 SH irradiance."""

    def __init__(self) -> None:
        super().__init__()
        self.coefficients = th.nn.Parameter(th.empty(1, 3, 9))
        with th.no_grad():
            self.coefficients.uniform_(-0.1, 0.1)
            self.coefficients[..., 0] = 0.5

    def forward(self, normals, diffuse):
        M = _sh_matrix(self.coefficients).view(1, 1, 3, 4, 4)
        n = th.cat([normals, th.ones_like(normals[..., :1])], dim=-1).view(normals.shape[0], normals.shape[1], 1, 1, 4)
        image = dot(n @ M, n, False)
        return diffuse * image.squeeze(-1) / math.pi


class DeferredSphericalHaromic(th.nn.Module):
    """shading.py:61-76: per-pixel SH shading through the CUDA op."""

    def __init__(self, batched=1) -> None:
        super().__init__()
        self.coefficients = th.nn.Parameter(th.empty(batched, 3, 9))
        with th.no_grad():
            self.coefficients.uniform_(-0.1, 0.1)
            self.coefficients[..., 0] = 0.5

    def forward(self, normals, diffuse):
        return SphericalHarmonicShading.apply(self.coefficients, normals, diffuse)


def _fusable(attribute: th.Tensor, camPoints: th.Tensor) -> bool:
    return (isinstance(attribute, th.Tensor) and attribute.is_cuda and attribute.dtype == th.float32
            and attribute.device == camPoints.device and attribute.dim() == 3
            and attribute.shape[1] == camPoints.shape[1] and attribute.shape[0] in (1, camPoints.shape[0]))


def _normalizeNormals(normals: th.Tensor) -> th.Tensor:
    norms = normals.norm(dim=-1, keepdim=True)
    normals = th.where(norms < 0.01, th.ones_like(normals), normals)
    return normalize(normals)


class Splatting(th.nn.Module):
    """render.py:230-376.  ``opts`` needs ``forward``, ``numSamples``,
    ``precision``, ``shadingMode`` (a RenderOptions or the reference's argparse
    namespace); ``sample_kwargs`` are passed to the sampler (``seed``,
    ``uniforms``, ``h``)."""

    def __init__(self, opts, logger, width: int, height: int, focallength: float, zmin: float, zmax: float,
                 smoothing: float) -> None:
        super().__init__()
        self.logger = logger
        self.width, self.height, self.focallength = int(width), int(height), float(focallength)
        self.coordForward = getattr(opts, "forward", "-z")
        self.smoothing = float(smoothing)
        self.numSamples = int(opts.numSamples)
        self.precision = float(opts.precision)
        self.shadingMode = opts.shadingMode
        self.affineTransform = AffineTransform.apply
        self.linearTransform = LinearTransform.apply
        self.backface = BackfaceCulling()
        self.sampling = FmmSampling()
        self.ewa = EWASplatting.apply
        self.depthBlending = DepthFiltering.apply
        self.linearInterpolation = LinearInterpolation.apply
        self.deferredShading = DiffuseShading.apply
        self.forwardShading = Lambert()
        self.sphericalHarmonics = DeferredSphericalHaromic()
        self.forwardHarmonics = ForwardSphericalHaromic()
        self.sample_kwargs = {}
        # per-splat shading modes run the fused render kernels (False: the
        # separate EWA / compositing / interpolation ops, same results)
        self.fused = True
        self._indices = None

    @property
    def indices(self):
        return None if self._indices is None else self._indices.cpu().clone()

    def forward(self, camPositions, camOrientations, pointPositions, pointNormals, pointStdDevs, pointDiffuse,
                ambientLight, lampDirections, lampIntensities, alpha=None):
        transformMatrix = world2Camera(camPositions, camOrientations)
        transformMatrix = transformForward(transformMatrix, self.coordForward).squeeze(1).contiguous()
        camPoints = self.affineTransform(transformMatrix, pointPositions)
        camNormals = self.linearTransform(transformMatrix, pointNormals)
        harmonics = self.shadingMode in ("sphericalHarmonics", "forwardHarmonics")
        flipped, backfaceNormals = self.backface(pointNormals if harmonics else None, camNormals)
        if harmonics:
            pointNormals = flipped
        with th.no_grad():
            indices = self.sampling(self.width, self.height, self.focallength, camPoints.detach(),
                                    backfaceNormals.detach().contiguous(), pointDiffuse, pointStdDevs.detach(),
                                    self.numSamples, self.smoothing, self.precision, **self.sample_kwargs)
        self._indices = indices
        camLampDirections = self.linearTransform(transformMatrix, lampDirections)
        # the modes that interpolate one per-splat attribute
        perSplat = None
        if self.shadingMode == "forward":
            perSplat = self.forwardShading(ambientLight, camLampDirections, lampIntensities, camNormals, pointDiffuse)
        elif self.shadingMode == "forwardHarmonics":
            perSplat = self.forwardHarmonics(pointNormals, pointDiffuse)
        elif self.shadingMode == "None":
            perSplat = pointDiffuse
        if perSplat is not None and self.fused and _fusable(perSplat, camPoints):
            # EWA -> compositing -> interpolation in one kernel each way
            image, depthWeights, _ = th.ops.uds.render_splats(
                self.width, self.height, self.focallength, indices, camPoints.contiguous(), camNormals.contiguous(),
                pointStdDevs.contiguous(), self.smoothing, perSplat.contiguous())
            return image, indices, depthWeights
        ewaWeights = self.ewa(self.width, self.height, self.focallength, indices, camPoints, camNormals, pointStdDevs,
                              self.smoothing)
        depthWeights = self.depthBlending(indices, ewaWeights, self.width, self.height, self.focallength, camPoints,
                                          camNormals)
        if self.shadingMode == "deferred":
            ewaNormals = _normalizeNormals(self.linearInterpolation(indices, depthWeights, camNormals))
            ewaDiffuse = self.linearInterpolation(indices, depthWeights, pointDiffuse)
            image = self.deferredShading(camLampDirections, lampIntensities, ewaNormals.contiguous(), ewaDiffuse)
        elif perSplat is not None:
            image = self.linearInterpolation(indices, depthWeights, perSplat)
        elif self.shadingMode == "sphericalHarmonics":
            ewaNormals = self.linearInterpolation(indices, depthWeights, pointNormals)
            ewaDiffuse = self.linearInterpolation(indices, depthWeights, pointDiffuse)
            image = self.sphericalHarmonics(ewaNormals, ewaDiffuse)
        elif self.shadingMode == "silhouette":
            image = th.clamp(th.sum(ewaWeights, dim=-1, keepdim=True), 0, 1)
        else:
            raise ValueError("Unkown shading mode")
        return image, indices, depthWeights


class MultiViewSplatting(th.nn.Module):
    """Splatting.forward for B views of different sizes in one pass (no
    counterpart module in the reference, which renders one view size per
    module): the transforms and back-face flips of all views at once, one
    sampling call whose descent covers every view's pixels in one launch
    (``sampling.sample_views``), then the fused render pass once per run of
    consecutive views of one size.  ``views`` lists (width, height,
    focallength) per view.  The shading modes that interpolate one per-splat
    attribute are supported: forward, forwardHarmonics, None.

    forward(...) takes Splatting.forward's arguments for all B views and
    returns (images, indices, depthWeights): lists with one (1,W_b,H_b,.)
    tensor per view."""

    MODES = ("forward", "forwardHarmonics", "None")

    def __init__(self, opts, logger, views, zmin: float, zmax: float, smoothing: float) -> None:
        super().__init__()
        if opts.shadingMode not in self.MODES:
            raise ValueError(f"MultiViewSplatting interpolates per-splat attributes ({', '.join(self.MODES)}); "
                             f"use one Splatting per view size for shading mode {opts.shadingMode!r}")
        self.views = [(int(w), int(h), float(f)) for (w, h, f) in views]
        self.coordForward = getattr(opts, "forward", "-z")
        self.smoothing = float(smoothing)
        self.numSamples = int(opts.numSamples)
        self.precision = float(opts.precision)
        self.shadingMode = opts.shadingMode
        self.backface = BackfaceCulling()
        self.forwardShading = Lambert()
        self.forwardHarmonics = ForwardSphericalHaromic()
        self.sample_kwargs = {}
        # runs of consecutive views of one size: (first view, count, W, H, f)
        self.groups = []
        for b, v in enumerate(self.views):
            if self.groups and self.groups[-1][2:] == v and self.groups[-1][0] + self.groups[-1][1] == b:
                g = self.groups[-1]
                self.groups[-1] = (g[0], g[1] + 1, *v)
            else:
                self.groups.append((b, 1, *v))

    def forward(self, camPositions, camOrientations, pointPositions, pointNormals, pointStdDevs, pointDiffuse,
                ambientLight, lampDirections, lampIntensities):
        from .cudaExtensions import sampling
        transformMatrix = world2Camera(camPositions, camOrientations)
        transformMatrix = transformForward(transformMatrix, self.coordForward).squeeze(1).contiguous()
        camPoints = AffineTransform.apply(transformMatrix, pointPositions)
        camNormals = LinearTransform.apply(transformMatrix, pointNormals)
        harmonics = self.shadingMode == "forwardHarmonics"
        flipped, backfaceNormals = self.backface(pointNormals if harmonics else None, camNormals)
        with th.no_grad():
            packed = sampling.sample_views(self.views, camPoints.detach(), backfaceNormals.detach().contiguous(),
                                           None, pointStdDevs.detach(), self.numSamples, self.smoothing,
                                           self.precision, **self.sample_kwargs)
        camLampDirections = LinearTransform.apply(transformMatrix, lampDirections)
        if self.shadingMode == "forward":
            perSplat = self.forwardShading(ambientLight, camLampDirections, lampIntensities, camNormals, pointDiffuse)
        elif harmonics:
            perSplat = self.forwardHarmonics(flipped, pointDiffuse)
        else:
            perSplat = pointDiffuse
        B = camPoints.shape[0]
        images, indices, depth = [], [], []
        for (b0, nb, W, H, f) in self.groups:
            sl = slice(b0, b0 + nb)
            # consecutive views of one size are consecutive in the packed buffer
            K = self.numSamples
            idx = packed[b0].as_strided((nb, W, H, K), (W * H * K, H * K, K, 1))
            sd = pointStdDevs if pointStdDevs.shape[0] == 1 else pointStdDevs[sl]
            attr = perSplat if perSplat.shape[0] == 1 and B > 1 else perSplat[sl]
            img, dw, _ = th.ops.uds.render_splats(W, H, f, idx, camPoints[sl].contiguous(),
                                                  camNormals[sl].contiguous(), sd.contiguous(), self.smoothing,
                                                  attr.contiguous())
            for k in range(nb):
                images.append(img[k:k + 1])
                indices.append(idx[k:k + 1])
                depth.append(dw[k:k + 1])
        return images, indices, depth
