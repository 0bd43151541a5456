"""Learned proposal for the stochastic sampling mode (no reference
counterpart).

A small network (16 features -> 64 -> 64 -> 64 -> 2 branch logits, bf16
operands with fp32 accumulation on the tensor cores, see ``uds_mlp_*`` in
include/uds.h) proposes, at each internal node of the FMM tree, the
probability q of descending left.  Each draw's importance weight is
``(leaf Gaussian / root FGT mass) / q_path``, so weighted estimates
``mean_k w_k f(j_k)`` are unbiased for ``sum_j p_j f(j)`` whatever the network
outputs (q > 0 on every branch), and the network only decides the variance.
It is trained on rows that the stochastic sampler produces itself: at every
node it visits, the features and the exact FGT branch probability
``m_left / (m_left + m_right)``.  Pixels whose effective sample size falls
below ``ess_tau * K`` are redrawn by the plain stochastic sampler.
"""
from __future__ import annotations

import torch

from ._lib import SampleParams, Workspace, check, load, need, ptr, stream_ptr  # noqa: F401
from .cudaExtensions import sampling

LAYERS = ((64, 16), (64, 64), (64, 64), (16, 64))  # (out, in); the last layer's rows 2..15 are zero


def param_count() -> int:
    return int(load().uds_mlp_param_count())


def init_params(seed: int = 0, device="cuda") -> torch.Tensor:
    """He-initialised flat parameter vector (W1, b1, ..., W4, b4)."""
    g = torch.Generator().manual_seed(seed)
    parts = []
    for out, inp in LAYERS:
        W = torch.randn(out, inp, generator=g) * (2.0 / inp) ** 0.5
        b = torch.zeros(out)
        if out == 16:
            W[2:] = 0
        parts += [W.reshape(-1), b]
    P = torch.cat(parts)
    assert P.numel() == param_count()
    return P.to(device)


class ProposalNet:
    """Parameters + Adam state of the proposal network, trained and
    evaluated by the library's tensor-core kernels."""

    def __init__(self, device="cuda", seed: int = 0):
        self.device = torch.device(device)
        self.params = init_params(seed, self.device)
        self.m1 = torch.zeros_like(self.params)
        self.m2 = torch.zeros_like(self.params)
        self.grad = torch.zeros_like(self.params)
        self.steps = 0
        self._err = torch.zeros(1, dtype=torch.int32, device=self.device)

    def logits(self, X: torch.Tensor) -> torch.Tensor:
        X = need(X, "features", device=self.device)
        out = torch.empty((X.shape[0], 2), device=self.device)
        check(load().uds_mlp_forward(X.shape[0], ptr(X), ptr(self.params), ptr(out), ptr(self._err),
                                     stream_ptr(self.device)), "mlp forward")
        return out

    def train(self, X: torch.Tensor, target: torch.Tensor, steps: int = 400, batch: int = 32768, lr: float = 3e-3,
              seed: int = 0):
        """Adam on the mean cross-entropy between softmax(logits) and
        (target, 1 - target); returns the loss of each step (a device tensor)."""
        X = need(X, "features", device=self.device)
        target = need(target, "target", device=self.device)
        L = load()
        s = stream_ptr(self.device)
        g = torch.Generator(device=self.device).manual_seed(seed)
        losses = torch.zeros(steps, device=self.device)
        n = X.shape[0]
        nb = min(batch, n)
        ws = Workspace.get(self.device, L.uds_mlp_grad_workspace_size(nb), "mlp_grad")
        for i in range(steps):
            sel = torch.randint(0, n, (nb,), device=self.device, generator=g)
            xb, tb = X[sel].contiguous(), target[sel].contiguous()
            check(L.uds_mlp_grad(xb.shape[0], ptr(xb), ptr(tb), ptr(self.params), ptr(self.grad), ptr(losses[i:]),
                                 ptr(self._err), ptr(ws), ws.numel(), s), "mlp grad")
            self.steps += 1
            check(L.uds_mlp_adam(ptr(self.params), ptr(self.grad), ptr(self.m1), ptr(self.m2), self.steps, lr, 0.9,
                                 0.999, 1e-8, s), "mlp adam")
        return losses

    def failed(self) -> bool:
        return bool(self._err.item())


def dataset(width, height, focallength, points, normals, stdDevs, smoothing, precision, stride=4, draws=8,
            cap=2_000_000, seed=0):
    """(features (R,16), target (R,)) from stochastic descents on view 0, in
    a fixed order (sorted by pixel, draw and depth), at most cap rows (the
    first rows of that order when there are more)."""
    tree = sampling.build_tree(width, height, focallength, points[:1], normals[:1], stdDevs[:1], 8, smoothing,
                               precision)
    prm, ws = tree["_prm"], tree["_ws"]
    prm.seed = int(seed)
    dev = points.device
    room = cap
    while True:
        X = torch.empty((room, 16), device=dev)
        t = torch.empty(room, device=dev)
        keys = torch.empty(room, dtype=torch.int64, device=dev)
        count = torch.zeros(1, dtype=torch.int32, device=dev)
        check(load().uds_proposal_dataset(prm, stride, draws, ptr(X), ptr(t), ptr(keys), ptr(count), room, ptr(ws),
                                          ws.numel(), stream_ptr(dev)), "proposal dataset")
        n = int(count.item())
        if n <= room:
            break
        room = n  # every row kept, so that the order (and the cut at cap) is fixed
    order = torch.argsort(keys[:n])[:cap]
    return X[order], t[order]


def sample(width, height, focallength, points, normals, stdDevs, numSamples, smoothing, precision, net=None,
           ess_tau=0.5, seed=None, h=None, return_stats=False):
    """K weighted draws per pixel: (indices (B,W,H,K) int32, weights
    (B,W,H,K) float32, fallback (B,W,H) bool, n_fallback (B,) int32).  With
    net None every pixel uses the stochastic sampler."""
    sampling._check(points, normals, stdDevs)
    dev = points.device
    B, K = points.shape[0], int(numSamples)
    if seed is None:
        seed = int(torch.randint(0, 2 ** 62, (1,)).item())
    prm = sampling.params(width, height, focallength, points, stdDevs, K, smoothing, precision, seed)
    L = load()
    nbytes = L.uds_proposal_workspace_size(prm)
    if nbytes == 0:
        raise ValueError("invalid sampling parameters")
    ws = Workspace.get(dev, nbytes, "proposal")
    idx = torch.empty((B, int(width), int(height), K), dtype=torch.int32, device=dev)
    w = torch.empty((B, int(width), int(height), K), device=dev)
    fb = torch.empty((B, int(width), int(height)), dtype=torch.uint8, device=dev)
    nfb = torch.zeros(B, dtype=torch.int32, device=dev)
    stats = torch.empty((B, 8), device=dev) if return_stats else None
    if h is not None:
        need(h, "h", device=dev)
    check(L.uds_sample_proposal(prm, ptr(points), ptr(normals), ptr(stdDevs), ptr(h),
                                ptr(net.params) if net is not None else None, float(ess_tau), ptr(idx), ptr(w),
                                ptr(fb), ptr(nfb), ptr(stats), ptr(ws), ws.numel(), stream_ptr(dev)),
          "proposal sample")
    if return_stats:
        return idx, w, fb.bool(), nfb, sampling.view_stats(stats)
    return idx, w, fb.bool(), nfb


def estimate(indices, weights, values):
    """Weighted Monte-Carlo estimate mean_k w_k values[j_k] per pixel:
    indices/weights (B,W,H,K), values (B|1, N, C) -> (B,W,H,C)."""
    B, W, H, K = indices.shape
    vals = values if values.shape[0] == B else values.expand(B, -1, -1)
    safe = indices.clamp_min(0).long().reshape(B, -1)
    g = torch.gather(vals, 1, safe[..., None].expand(-1, -1, vals.shape[2])).reshape(B, W, H, K, -1)
    wk = torch.where(indices >= 0, weights, torch.zeros_like(weights))[..., None]
    return (g * wk).sum(3) / K
