"""Nearest-sample regulariser with the interface of the reference's
``NearestSamplesRegularizer`` (splatting/regularizier.py:119-175).

For every splat the neighbours are the splats sampled together with it in
the pixels where it is the surface sample (``nearestsamples.nearest``).  Two
losses pull the surface together: the plane loss, the squared weighted mean
distance of the splat from its neighbours' tangent planes, and the normal
loss, the squared distance of the splat's normal from its neighbours'
weighted mean normal; neighbour weights are Gaussians of the point and normal
distances with width ``sigma``.  Both losses and their gradients come from
one CUDA kernel over the neighbour lists (``nearestsamples.regularizer``);
as in the reference, the weights, the neighbours and the mean normals are
constants of the loss, and neighbour index 0 is masked.
"""
from __future__ import annotations

import torch as th

from .cudaExtensions import nearestsamples

REDUCTIONS = ("sum", "mean")


class _NearestLosses(th.autograd.Function):
    @staticmethod
    def forward(ctx, points, normals, nearest, sigma, mean):
        losses, gp, gn = nearestsamples.regularizer(nearest, points.detach().contiguous(),
                                                    normals.detach().contiguous(), sigma, mean)
        ctx.save_for_backward(gp, gn)
        return losses[0], losses[1]

    @staticmethod
    def backward(ctx, g_normal, g_plane):
        gp, gn = ctx.saved_tensors
        return gp * g_plane, gn * g_normal, None, None, None


class NearestSamplesRegularizer(th.nn.Module):
    """forward(indices, weights, points, normals) -> (normal loss, plane loss),
    summed over splats ("sum") or averaged ("mean")."""

    def __init__(self, sigma=0.5, num_nearest=10, reduction="sum") -> None:
        super().__init__()
        self.sigma = sigma
        self.num_nearest = num_nearest
        self.reduction = reduction
        self.nearest = nearestsamples.nearest

    def forward(self, indices, weights, points, normals):
        if self.reduction not in REDUCTIONS:
            raise ValueError(f"unknown reduction mode {self.reduction!r}")
        with th.no_grad():
            nearest = self.nearest(indices, weights.detach().contiguous(), points.detach().contiguous(),
                                   self.num_nearest)
        return _NearestLosses.apply(points, normals, nearest, float(self.sigma), self.reduction == "mean")
