"""Nearest-sample regulariser (splatting/regularizier.py:119-175), on top of
``cudaExtensions.nearestsamples.nearest``.

For every splat the neighbours come from the pixels where it is the surface
sample; the regulariser pulls each splat towards the planes of its
neighbours (plane loss) and its normal towards their weighted mean normal
(normal loss), with Gaussian weights on point and normal distances.  The
formula is the reference's, including its mask ``nearest > 0`` (which also
drops neighbour index 0).
"""
from __future__ import annotations

import torch as th

from .cudaExtensions import nearestsamples
from .extensions import normalize


def _dot(a, b):
    return th.sum(a * b, dim=-1, keepdim=True)


class NearestSamplesRegularizer(th.nn.Module):
    def __init__(self, sigma=0.5, num_nearest=10, reduction="sum") -> None:
        super().__init__()
        self.sigma = sigma
        self.num_nearest = num_nearest
        self.reduction = reduction
        self.nearest = nearestsamples.nearest

    def _gaussian(self, x):
        return th.exp(-x.square() / self.sigma ** 2)

    def forward(self, indices, weights, points, normals):
        with th.no_grad():
            nearestIndices = self.nearest(indices, weights.contiguous(), points.detach().contiguous(),
                                          self.num_nearest)
            mask = (nearestIndices > 0).to(points.dtype).unsqueeze(-1)
            nearestIndices = nearestIndices.clamp(0)
            nearestPoints = points[0, nearestIndices[0].long(), :].unsqueeze(0)
            nearestNormals = normals[0, nearestIndices[0].long(), :].unsqueeze(0)
            anisotropic = (normals.unsqueeze(2) - nearestNormals).norm(dim=-1, keepdim=True)
            isotropic = (points.unsqueeze(2) - nearestPoints.detach()).norm(dim=-1, keepdim=True)
            w = mask * self._gaussian(anisotropic) * self._gaussian(isotropic)
            invWeights = 1.0 / (w.sum(dim=2) + 1e-4)
            filteredNormals = normalize(th.sum(w * nearestNormals, dim=2))
            pixelMask = mask.sum(dim=2).clamp(0, 1)
        planeDistance = w.detach() * _dot(points.unsqueeze(2) - nearestPoints.detach(), nearestNormals.detach())
        planeLoss = th.square(invWeights.detach() * planeDistance.sum(dim=2))
        normalDistance = th.square(filteredNormals.detach() - normals).sum(dim=-1, keepdim=True)
        normalLoss = pixelMask.detach() * normalDistance
        if self.reduction == "sum":
            return normalLoss.sum(), planeLoss.sum()
        if self.reduction == "mean":
            return normalLoss.mean(), planeLoss.mean()
        raise ValueError("Unkown reduction mode")
