"""Fused training-step tail for splat optimisation (the loop of
optimization_geometry.py:150-219): image losses that produce their gradient
in the same pass (``L1ImageLoss``, ``L2ImageLoss`` with the reference's
names and reductions), and ``SplatAdam``, one kernel launch per step for
Adam over positions, normals, colours and std-devs followed by the loop's
constraint projection (normals renormalised, std-devs clamped)."""
from __future__ import annotations

import torch as th

from ._lib import check, load, need, ptr, stream_ptr


class _FusedImageLoss(th.autograd.Function):
    @staticmethod
    def forward(ctx, kind, scale, x, y):
        x = need(x.contiguous(), "image")
        y = need(y.contiguous(), "target", device=x.device)
        loss = th.empty((), device=x.device)
        grad = th.empty_like(x)
        check(load().uds_image_loss(kind, x.numel(), ptr(x), ptr(y), float(scale), ptr(loss), ptr(grad),
                                    stream_ptr(x.device)), "image loss")
        ctx.save_for_backward(grad)
        return loss

    @staticmethod
    def backward(ctx, g):
        (grad,) = ctx.saved_tensors
        return None, None, grad * g, None


class _ImageLoss(th.nn.Module):
    kind = 0

    def __init__(self, reduction: str = "mean") -> None:
        super().__init__()
        if reduction not in ("mean", "sum"):
            raise ValueError("Unkown reduction mode")
        self.reduction = reduction

    def forward(self, x, y):
        scale = 1.0 / x.numel() if self.reduction == "mean" else 1.0
        return _FusedImageLoss.apply(self.kind, scale, x, y), None


class L1ImageLoss(_ImageLoss):
    """losses.py:19-31 (returns (loss, None) like the reference)."""
    kind = 0


class L2ImageLoss(_ImageLoss):
    """losses.py:5-17."""
    kind = 1


class SplatAdam:
    """Adam (torch defaults: no weight decay, no amsgrad) over the splat
    tensors (1, N, c) points, normals, colors, stdDevs, with the reference
    loop's projection after the step; one kernel launch per step."""

    def __init__(self, points, normals, colors, stdDevs, lr=1e-3, betas=(0.9, 0.999), eps=1e-8,
                 stdDevBound=(0.0, float("inf")), project=True):
        self.tensors = [points, normals, colors, stdDevs]
        self.N = points.shape[1]
        self.C = colors.shape[2] if colors is not None else 0
        width = 3 + 3 + self.C + 2
        dev = points.device
        self.m = th.zeros(self.N * width, device=dev)
        self.v = th.zeros(self.N * width, device=dev)
        self.lr, self.betas, self.eps = lr, betas, eps
        self.bounds = stdDevBound
        self.project = project
        self.steps = 0

    def zero_grad(self, set_to_none=True):
        for t in self.tensors:
            if t is not None and t.grad is not None:
                if set_to_none:
                    t.grad = None
                else:
                    t.grad.zero_()

    @th.no_grad()
    def step(self):
        self.steps += 1
        p = [t.data if t is not None else None for t in self.tensors]
        g = [t.grad.contiguous() if (t is not None and t.grad is not None) else None for t in self.tensors]
        dev = self.tensors[0].device
        check(load().uds_adam_splats(self.N, ptr(p[0]), ptr(g[0]), ptr(p[1]), ptr(g[1]), ptr(p[2]), ptr(g[2]),
                                     self.C, ptr(p[3]), ptr(g[3]), ptr(self.m), ptr(self.v), self.steps, self.lr,
                                     self.betas[0], self.betas[1], self.eps, float(self.bounds[0]),
                                     float(self.bounds[1]), int(self.project), stream_ptr(dev)), "adam splats")
