"""The CUDA ops registered with PyTorch's dispatcher as ``torch.ops.uds.*``.

Each op is a ``torch.library.custom_op`` over the C-ABI wrapper of
``cudaExtensions`` (the reference's pybind entry points: sampling.cpp:177-183,
splatting.cpp:131-136, zSorting.cpp:45-49, interpolation.cpp, shading.cpp,
transform.cpp), with a fake (meta) implementation for shape propagation, and
the differentiable ones with their backward op registered as autograd
formula, so that ``torch.compile`` traces a render without graph breaks and
``torch.library.opcheck`` can check every op.  The gradients registered here
are the kernels' raw gradients, except ``ewa_weights``: the EWA weights with
the reference's post-processing of their gradient (norm clamp, NaN scrub,
dropped normal gradient), which ``extensions.EWASplatting`` and the renderer
use.

Schemas use the reference's argument order; names are snake_case
(``splat_forward`` for ``splatting.forward``).
"""
from __future__ import annotations

from typing import List, Optional, Tuple

import torch
from torch import Tensor

from .cudaExtensions import (filtering, interpolation, nearestsamples, pixelgather, sampling, shading, splatting,
                             transform)

_op = torch.library.custom_op


# ---------------------------------------------------------------- sampling
@_op("uds::sample", mutates_args=())
def sample(width: int, height: int, focallength: float, points: Tensor, normals: Tensor, stdDevs: Tensor,
           numSamples: int, smoothing: float, precision: float, seed: int, seed_tensor: Optional[Tensor],
           uniforms: Optional[Tensor], leaf_size: int = 0) -> Tensor:
    """sampling.sample: (B,W,H,K) int32 splat indices.  The Philox key is
    ``seed_tensor`` (one int64 on the device, read when the kernels run) when
    given, else ``seed``; ``uniforms`` (B,W,H,R,max(K,leaf_size)) replaces the
    generator."""
    return sampling.sample(width, height, focallength, points, normals, None, stdDevs, numSamples, smoothing,
                           precision, uniforms=uniforms, seed=seed_tensor if seed_tensor is not None else seed,
                           leaf_size=leaf_size)


@sample.register_fake
def _(width, height, focallength, points, normals, stdDevs, numSamples, smoothing, precision, seed, seed_tensor,
      uniforms, leaf_size=0):
    return points.new_empty((points.shape[0], width, height, numSamples), dtype=torch.int32)


@_op("uds::sample_views", mutates_args=())
def sample_views(widths: List[int], heights: List[int], focallengths: List[float], points: Tensor, normals: Tensor,
                 stdDevs: Tensor, numSamples: int, smoothing: float, precision: float, seed: int,
                 seed_tensor: Optional[Tensor], leaf_size: int = 0) -> List[Tensor]:
    """Views of different sizes in one call: [(1,W_b,H_b,K) int32 per view]."""
    views = list(zip(widths, heights, focallengths))
    out = sampling.sample_views(views, points, normals, None, stdDevs, numSamples, smoothing, precision,
                                seed=seed_tensor if seed_tensor is not None else seed, leaf_size=leaf_size)
    return [t.clone() for t in out]


@sample_views.register_fake
def _(widths, heights, focallengths, points, normals, stdDevs, numSamples, smoothing, precision, seed, seed_tensor,
      leaf_size=0):
    return [points.new_empty((1, w, h, numSamples), dtype=torch.int32) for w, h in zip(widths, heights)]


# --------------------------------------------------------------------- EWA
@_op("uds::splat_forward", mutates_args=())
def splat_forward(width: int, height: int, focallength: float, indices: Tensor, points: Tensor, normals: Tensor,
                  stdDevs: Tensor, smoothing: float) -> Tensor:
    return splatting.forward(width, height, focallength, indices, points, normals, stdDevs, smoothing)


@splat_forward.register_fake
def _(width, height, focallength, indices, points, normals, stdDevs, smoothing):
    return points.new_empty(indices.shape)


@_op("uds::splat_backward", mutates_args=())
def splat_backward(width: int, height: int, focallength: float, gradIn: Tensor, indices: Tensor, points: Tensor,
                   normals: Tensor, stdDevs: Tensor, smoothing: float) -> Tuple[Tensor, Tensor, Tensor]:
    gp, gn, gs = splatting.backward(width, height, focallength, gradIn, indices, points, normals, stdDevs, smoothing)
    return gp, gn, gs


@splat_backward.register_fake
def _(width, height, focallength, gradIn, indices, points, normals, stdDevs, smoothing):
    return torch.empty_like(points), torch.empty_like(normals), torch.empty_like(stdDevs)


def _splat_setup(ctx, inputs, output):
    width, height, focallength, indices, points, normals, stdDevs, smoothing = inputs
    ctx.save_for_backward(indices, points, normals, stdDevs)
    ctx.args = (width, height, focallength, smoothing)


def _splat_grad(ctx, grad):
    indices, points, normals, stdDevs = ctx.saved_tensors
    width, height, focallength, smoothing = ctx.args
    gp, gn, gs = torch.ops.uds.splat_backward(width, height, focallength, grad.contiguous(), indices, points,
                                              normals, stdDevs, smoothing)
    return None, None, None, None, gp, gn, gs, None


splat_forward.register_autograd(_splat_grad, setup_context=_splat_setup)


@_op("uds::ewa_weights", mutates_args=())
def ewa_weights(width: int, height: int, focallength: float, indices: Tensor, points: Tensor, normals: Tensor,
                stdDevs: Tensor, smoothing: float) -> Tensor:
    """EWASplatting (extensions/__init__.py:175-233): the weights of
    splat_forward with the reference's gradient conventions: each splat's
    point and std-dev gradient scaled to norm <= 1 (conditionalNormalization,
    utils.py:147-150), NaNs set to 0, no gradient for the normals."""
    return splatting.forward(width, height, focallength, indices, points, normals, stdDevs, smoothing)


@ewa_weights.register_fake
def _(width, height, focallength, indices, points, normals, stdDevs, smoothing):
    return points.new_empty(indices.shape)


def _clamp_rows(dx: Tensor, eps: float = 1e-4) -> Tensor:
    return dx / torch.clamp(dx.norm(dim=-1, keepdim=True) + eps, 1.0)


def _ewa_grad(ctx, grad):
    indices, points, normals, stdDevs = ctx.saved_tensors
    width, height, focallength, smoothing = ctx.args
    gp, _, gs = torch.ops.uds.splat_backward(width, height, focallength, grad.contiguous(), indices, points, normals,
                                             stdDevs, smoothing)
    gp = torch.nan_to_num(_clamp_rows(gp), nan=0.0, posinf=float("inf"), neginf=float("-inf"))
    gs = torch.nan_to_num(_clamp_rows(gs), nan=0.0, posinf=float("inf"), neginf=float("-inf"))
    return None, None, None, None, gp, None, gs, None


ewa_weights.register_autograd(_ewa_grad, setup_context=_splat_setup)


@_op("uds::render_splats", mutates_args=())
def render_splats(width: int, height: int, focallength: float, indices: Tensor, points: Tensor, normals: Tensor,
                  stdDevs: Tensor, smoothing: float, attribute: Tensor) -> Tuple[Tensor, Tensor, Tensor]:
    """EWA weights -> depth compositing -> interpolation of the per-splat
    attribute (1|B,N,C) in one fused pass: (image (B,W,H,C), depth weights,
    EWA weights), bit-identical to ewa_weights, filter_forward and
    interp_forward.  Gradients as that chain: the EWA part with the
    reference's post-processing (ewa_weights), none for the normals."""
    image, depth, weights = splatting.renderForward(width, height, focallength, indices, points, normals, stdDevs,
                                                    smoothing, attribute)
    return image, depth, weights


@render_splats.register_fake
def _(width, height, focallength, indices, points, normals, stdDevs, smoothing, attribute):
    B, W, H, _ = indices.shape
    return (points.new_empty((B, W, H, attribute.shape[2])), points.new_empty(indices.shape),
            points.new_empty(indices.shape))


@_op("uds::render_splats_backward", mutates_args=())
def render_splats_backward(width: int, height: int, focallength: float, gradImage: Tensor,
                           gradDepthWeights: Optional[Tensor], gradWeights: Optional[Tensor], indices: Tensor,
                           weights: Tensor, points: Tensor, normals: Tensor, stdDevs: Tensor, smoothing: float,
                           attribute: Tensor) -> List[Tensor]:
    """Raw gradients of render_splats: [points, normals, std-devs, attribute]."""
    return splatting.renderBackward(width, height, focallength, gradImage, gradDepthWeights, gradWeights, indices,
                                    weights, points, normals, stdDevs, smoothing, attribute)


@render_splats_backward.register_fake
def _(width, height, focallength, gradImage, gradDepthWeights, gradWeights, indices, weights, points, normals,
      stdDevs, smoothing, attribute):
    return [torch.empty_like(t) for t in (points, normals, stdDevs, attribute)]


def _render_setup(ctx, inputs, output):
    width, height, focallength, indices, points, normals, stdDevs, smoothing, attribute = inputs
    ctx.save_for_backward(indices, points, normals, stdDevs, attribute, output[2])
    ctx.args = (width, height, focallength, smoothing)
    ctx.image_shape = output[0].shape


def _render_grad(ctx, g_image, g_depth, g_weights):
    indices, points, normals, stdDevs, attribute, weights = ctx.saved_tensors
    width, height, focallength, smoothing = ctx.args
    if g_image is None:
        g_image = weights.new_zeros(ctx.image_shape)
    c = lambda t: None if t is None else t.contiguous()  # noqa: E731
    gp, _, gs, ga = torch.ops.uds.render_splats_backward(width, height, focallength, g_image.contiguous(),
                                                         c(g_depth), c(g_weights), indices, weights, points,
                                                         normals, stdDevs, smoothing, attribute)
    gp = torch.nan_to_num(_clamp_rows(gp), nan=0.0, posinf=float("inf"), neginf=float("-inf"))
    gs = torch.nan_to_num(_clamp_rows(gs), nan=0.0, posinf=float("inf"), neginf=float("-inf"))
    return None, None, None, None, gp, None, gs, None, ga


render_splats.register_autograd(_render_grad, setup_context=_render_setup)


# ------------------------------------------------------------- compositing
@_op("uds::filter_forward", mutates_args=())
def filter_forward(indices: Tensor, weights: Tensor, width: int, height: int, focallength: float, points: Tensor,
                   normals: Tensor) -> Tensor:
    return filtering.forward(indices, weights, width, height, focallength, points, normals)


@filter_forward.register_fake
def _(indices, weights, width, height, focallength, points, normals):
    return torch.empty_like(weights)


@_op("uds::filter_backward", mutates_args=())
def filter_backward(indices: Tensor, weights: Tensor, gradIn: Tensor, width: int, height: int, focallength: float,
                    points: Tensor, normals: Tensor) -> Tensor:
    return filtering.backward(indices, weights, gradIn, width, height, focallength, points, normals)


@filter_backward.register_fake
def _(indices, weights, gradIn, width, height, focallength, points, normals):
    return torch.empty_like(weights)


def _filter_setup(ctx, inputs, output):
    indices, weights, width, height, focallength, points, normals = inputs
    ctx.save_for_backward(indices, weights, points, normals)
    ctx.args = (width, height, focallength)


def _filter_grad(ctx, grad):
    indices, weights, points, normals = ctx.saved_tensors
    width, height, focallength = ctx.args
    gw = torch.ops.uds.filter_backward(indices, weights, grad.contiguous(), width, height, focallength, points,
                                       normals)
    return None, gw, None, None, None, None, None


filter_forward.register_autograd(_filter_grad, setup_context=_filter_setup)


# ----------------------------------------------------------- interpolation
@_op("uds::interp_forward", mutates_args=())
def interp_forward(indices: Tensor, weights: Tensor, attribute: Tensor) -> Tensor:
    return interpolation.forward(indices, weights, attribute)


@interp_forward.register_fake
def _(indices, weights, attribute):
    B, W, H, _ = indices.shape
    return attribute.new_empty((B, W, H, attribute.shape[2]))


@_op("uds::interp_backward", mutates_args=())
def interp_backward(gradIn: Tensor, indices: Tensor, weights: Tensor, attribute: Tensor) -> Tuple[Tensor, Tensor]:
    gw, ga = interpolation.backward(gradIn, indices, weights, attribute)
    return gw, ga


@interp_backward.register_fake
def _(gradIn, indices, weights, attribute):
    return torch.empty_like(weights), torch.empty_like(attribute)


def _interp_setup(ctx, inputs, output):
    ctx.save_for_backward(*inputs)


def _interp_grad(ctx, grad):
    indices, weights, attribute = ctx.saved_tensors
    gw, ga = torch.ops.uds.interp_backward(grad.contiguous(), indices, weights, attribute)
    return None, gw, ga


interp_forward.register_autograd(_interp_grad, setup_context=_interp_setup)


# --------------------------------------------------------------- transform
def _transform_op(name, affine):
    fwd_name, bwd_name = f"uds::{name}_forward", f"uds::{name}_backward"
    fwd_impl = transform.affineForward if affine else transform.linearForward
    bwd_impl = transform.affineBackward if affine else transform.linearBackward

    @_op(fwd_name, mutates_args=())
    def fwd(transformation: Tensor, vector: Tensor) -> Tensor:
        return fwd_impl(transformation, vector)

    @fwd.register_fake
    def _(transformation, vector):
        return vector.new_empty((transformation.shape[0], vector.shape[1], 3))

    @_op(bwd_name, mutates_args=())
    def bwd(gradIn: Tensor, transformation: Tensor, vector: Tensor) -> Tuple[Tensor, Tensor]:
        gM, gv = bwd_impl(gradIn, transformation, vector)
        return gM, gv

    @bwd.register_fake
    def _(gradIn, transformation, vector):
        return torch.empty_like(transformation), torch.empty_like(vector)

    backward_op = getattr(torch.ops.uds, f"{name}_backward")

    def setup(ctx, inputs, output):
        ctx.save_for_backward(*inputs)

    def grad(ctx, g):
        M, v = ctx.saved_tensors
        gM, gv = backward_op(g.contiguous(), M, v)
        return gM, gv

    fwd.register_autograd(grad, setup_context=setup)
    return fwd, bwd


affine_forward, affine_backward = _transform_op("affine", True)
linear_forward, linear_backward = _transform_op("linear", False)


@_op("uds::view_matrix_forward", mutates_args=())
def view_matrix_forward(positions: Tensor, quaternions: Tensor) -> Tensor:
    """world2Camera: (B,3) positions, (B,4) quaternions (x,y,z,w) -> (B,1,4,4)."""
    return transform.viewMatrixForward(positions, quaternions)


@view_matrix_forward.register_fake
def _(positions, quaternions):
    return positions.new_empty((quaternions.shape[0], 1, 4, 4))


@_op("uds::view_matrix_backward", mutates_args=())
def view_matrix_backward(gradIn: Tensor, quaternions: Tensor) -> Tuple[Tensor, Tensor]:
    gp, gq = transform.viewMatrixBackward(gradIn, quaternions)
    return gp, gq


@view_matrix_backward.register_fake
def _(gradIn, quaternions):
    return quaternions.new_empty((quaternions.shape[0], 3)), torch.empty_like(quaternions)


def _view_setup(ctx, inputs, output):
    ctx.save_for_backward(inputs[1])


def _view_grad(ctx, grad):
    (q,) = ctx.saved_tensors
    gp, gq = torch.ops.uds.view_matrix_backward(grad.contiguous(), q)
    return gp, gq


view_matrix_forward.register_autograd(_view_grad, setup_context=_view_setup)


@_op("uds::backface", mutates_args=())
def backface(camNormals: Tensor, normals: Optional[Tensor]) -> List[Tensor]:
    """BackfaceCulling (render.py:193-205): [flipped camera-space normals]
    + [flipped world normals (B,N,3)] when ``normals`` is given."""
    return transform.backfaceForward(camNormals, normals)


@backface.register_fake
def _(camNormals, normals):
    return [torch.empty_like(camNormals)] + ([] if normals is None else [torch.empty_like(camNormals)])


@_op("uds::backface_backward", mutates_args=())
def backface_backward(camNormals: Tensor, gradCam: Tensor, gradNormals: Optional[Tensor],
                      normalsBatch: int) -> List[Tensor]:
    gc, gw = transform.backfaceBackward(camNormals, gradCam, gradNormals, normalsBatch)
    return [gc] if gw is None else [gc, gw]


@backface_backward.register_fake
def _(camNormals, gradCam, gradNormals, normalsBatch):
    out = [torch.empty_like(camNormals)]
    if gradNormals is not None:
        out.append(camNormals.new_empty((normalsBatch, camNormals.shape[1], 3)))
    return out


def _backface_setup(ctx, inputs, output):
    camNormals, normals = inputs
    ctx.save_for_backward(camNormals)
    ctx.normalsBatch = None if normals is None else normals.shape[0]


def _backface_grad(ctx, grads):
    (camNormals,) = ctx.saved_tensors
    gcam = grads[0] if grads[0] is not None else torch.zeros_like(camNormals)
    gnrm = None
    if ctx.normalsBatch is not None and len(grads) > 1 and grads[1] is not None:
        gnrm = grads[1].contiguous()
    out = torch.ops.uds.backface_backward(camNormals, gcam.contiguous(), gnrm, ctx.normalsBatch or 1)
    return out[0], (out[1] if gnrm is not None else None)


backface.register_autograd(_backface_grad, setup_context=_backface_setup)


# ----------------------------------------------------------------- shading
@_op("uds::shade_forward", mutates_args=())
def shade_forward(directions: Tensor, intensities: Tensor, normals: Tensor, diffuse: Tensor) -> Tensor:
    return shading.forward(directions, intensities, normals, diffuse)


@shade_forward.register_fake
def _(directions, intensities, normals, diffuse):
    return torch.empty_like(normals)


@_op("uds::shade_backward", mutates_args=())
def shade_backward(gradIn: Tensor, directions: Tensor, intensities: Tensor, normals: Tensor,
                   diffuse: Tensor) -> List[Tensor]:
    return shading.backward(gradIn, directions, intensities, normals, diffuse)


@shade_backward.register_fake
def _(gradIn, directions, intensities, normals, diffuse):
    return [torch.empty_like(t) for t in (directions, intensities, normals, diffuse)]


def _save_all(ctx, inputs, output):
    ctx.save_for_backward(*inputs)


def _shade_grad(ctx, grad):
    return tuple(torch.ops.uds.shade_backward(grad.contiguous(), *ctx.saved_tensors))


shade_forward.register_autograd(_shade_grad, setup_context=_save_all)


@_op("uds::shade_sh_forward", mutates_args=())
def shade_sh_forward(coefficients: Tensor, normals: Tensor, diffuse: Tensor) -> Tensor:
    return shading.forwardSh(coefficients, normals, diffuse)


@shade_sh_forward.register_fake
def _(coefficients, normals, diffuse):
    return torch.empty_like(normals)


@_op("uds::shade_sh_backward", mutates_args=())
def shade_sh_backward(gradIn: Tensor, coefficients: Tensor, normals: Tensor, diffuse: Tensor) -> List[Tensor]:
    return shading.backwardSh(gradIn, coefficients, normals, diffuse)


@shade_sh_backward.register_fake
def _(gradIn, coefficients, normals, diffuse):
    return [torch.empty_like(t) for t in (coefficients, normals, diffuse)]


def _shade_sh_grad(ctx, grad):
    return tuple(torch.ops.uds.shade_sh_backward(grad.contiguous(), *ctx.saved_tensors))


shade_sh_forward.register_autograd(_shade_sh_grad, setup_context=_save_all)


@_op("uds::lambert_forward", mutates_args=())
def lambert_forward(ambient: Tensor, directions: Tensor, intensities: Tensor, normals: Tensor,
                    diffuse: Tensor) -> Tensor:
    """Per-splat ambient + Lambert shading (shading.py:12-29) for the operand
    shapes of ``cudaExtensions.shading.lambert_shapes``."""
    return shading.lambertForward(ambient, directions, intensities, normals, diffuse)


@lambert_forward.register_fake
def _(ambient, directions, intensities, normals, diffuse):
    return torch.empty_like(normals)


@_op("uds::lambert_backward", mutates_args=())
def lambert_backward(gradIn: Tensor, ambient: Tensor, directions: Tensor, intensities: Tensor, normals: Tensor,
                     diffuse: Tensor) -> List[Tensor]:
    return shading.lambertBackward(gradIn, ambient, directions, intensities, normals, diffuse)


@lambert_backward.register_fake
def _(gradIn, ambient, directions, intensities, normals, diffuse):
    return [torch.empty_like(t) for t in (ambient, directions, intensities, normals, diffuse)]


def _lambert_grad(ctx, grad):
    return tuple(torch.ops.uds.lambert_backward(grad.contiguous(), *ctx.saved_tensors))


lambert_forward.register_autograd(_lambert_grad, setup_context=_save_all)


# ------------------------------------------------- per-splat consumers
@_op("uds::pixel_scatter", mutates_args=())
def pixel_scatter(indices: Tensor, values: Tensor) -> Tensor:
    return pixelgather.scatter(indices, values)


@pixel_scatter.register_fake
def _(indices, values):
    B, W, H, K = indices.shape
    return values.new_empty((B, W, H, K, values.shape[2]))


@_op("uds::pixel_gather", mutates_args=())
def pixel_gather(indices: Tensor, values: Tensor, numSources: int, deterministic: bool) -> Tensor:
    return pixelgather.gather(indices, values, numSources, deterministic)


@pixel_gather.register_fake
def _(indices, values, numSources, deterministic):
    return values.new_empty((indices.shape[0], numSources, values.shape[4]))


def _scatter_setup(ctx, inputs, output):
    indices, values = inputs
    ctx.save_for_backward(indices)
    ctx.numSources = values.shape[1]


def _scatter_grad(ctx, grad):
    (indices,) = ctx.saved_tensors
    return None, torch.ops.uds.pixel_gather(indices, grad.contiguous(), ctx.numSources, False)


pixel_scatter.register_autograd(_scatter_grad, setup_context=_scatter_setup)


@_op("uds::nearest", mutates_args=())
def nearest(indices: Tensor, weights: Tensor, points: Tensor, numNearest: int) -> Tensor:
    return nearestsamples.nearest(indices, weights, points, numNearest)


@nearest.register_fake
def _(indices, weights, points, numNearest):
    return points.new_empty((1, points.shape[1], numNearest), dtype=torch.int32)


@_op("uds::nearest_regularizer", mutates_args=())
def nearest_regularizer(nearest: Tensor, points: Tensor, normals: Tensor, sigma: float,
                        mean: bool) -> Tuple[Tensor, Tensor, Tensor]:
    losses, gp, gn = nearestsamples.regularizer(nearest, points, normals, sigma, mean)
    return losses, gp, gn


@nearest_regularizer.register_fake
def _(nearest, points, normals, sigma, mean):
    return points.new_empty((2,)), torch.empty_like(points), torch.empty_like(normals)


OPS = ("sample", "sample_views", "splat_forward", "splat_backward", "ewa_weights", "render_splats", "render_splats_backward", "filter_forward", "filter_backward", "interp_forward",
       "interp_backward", "affine_forward", "affine_backward", "linear_forward", "linear_backward",
       "view_matrix_forward", "view_matrix_backward", "backface", "backface_backward", "shade_forward", "shade_backward", "shade_sh_forward",
       "shade_sh_backward", "lambert_forward", "lambert_backward", "pixel_scatter", "pixel_gather", "nearest",
       "nearest_regularizer")
