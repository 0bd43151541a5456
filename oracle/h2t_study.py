"""Would a Hermite-to-Taylor (H2T) downward pass pay on this path?  A CPU
study on the headline view's tree (harmonic surface, 500k surfels, 1024^2,
precision 0.01), using the oracle's tree build.  Test infrastructure: it
only measures; nothing in the product imports it.

The FGT's downward pass (evaluateDynamicRadixTree.cuh:14-95,
hermitefmm.cuh:140-181, 240-256: the reference's Taylor stage, never filled
on its live path) converts far nodes' Hermite expansions into one Taylor
expansion about the centre of a cell of s x s pixels, evaluated at each of
the cell's pixels.  Two questions, with u = (pixel - cell centre)/sqrt(2) h
and a = (source - cell centre)/sqrt(2) h per axis:

1. Degree: the smallest Taylor degree q with which every source Gaussian
   exp(-(u - a)^2) (per axis; the 2-D error is at most about twice the 1-D
   one) is reproduced within 1e-4 absolute (1e-4 relative to a unit mass)
   for all pixels of the cell and all sources within the truncation radius
   of the cell's pixels.
2. Cost per pixel: the descent needs the mass of every node on its paths,
   not only the total, so each evaluated node needs its own Taylor
   expansion: per pixel (q+1)^2 terms per node instead of (p+1)^2, plus the
   conversion, (p+1)(q+1)(p+q+2) multiply-adds per node done separably by
   axis, shared by the cell's s^2 pixels.  Evaluated over the nodes a pixel
   actually evaluates (the frontier the root walk meets), for a sample of
   pixels.

    python oracle/h2t_study.py [--pixels 400]
"""
from __future__ import annotations

import argparse
import math
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)


def taylor_degree(s: int, a_max: float, tol: float = 1e-4, h: float = 1.0) -> int:
    """Smallest q with max |exp(-(u-a)^2) - T_q(u; a)| <= tol / 2 over the
    cell's pixel offsets u and |a| <= a_max (units of sqrt(2) h)."""
    offs = (np.arange(s) - (s - 1) / 2.0) / (math.sqrt(2.0) * h)
    a = np.linspace(-a_max, a_max, 2001)
    # exp(-(u-a)^2) = exp(-a^2) sum_n H_n(a) u^n / n!, H_n the physicists' Hermite polynomials
    for q in range(0, 80):
        Hn = [np.ones_like(a), 2 * a]
        for n in range(2, q + 1):
            Hn.append(2 * a * Hn[-1] - 2 * (n - 1) * Hn[-2])
        err = 0.0
        for u in offs:
            t = sum(Hn[n] * u ** n / math.factorial(n) for n in range(q + 1)) * np.exp(-a * a)
            err = max(err, float(np.max(np.abs(np.exp(-(u - a) ** 2) - t))))
        if 2 * err <= tol:
            return q
    return -1


def main():
    import torch
    import oracle
    from unbiased_differentiable_splatting_gb300 import scenes as S
    ap = argparse.ArgumentParser()
    ap.add_argument("--pixels", type=int, default=400)
    args = ap.parse_args()
    sc = S.harmonic_scene(n=500_000, sd_range=(0.003, 0.01), width=1024, seed=0)
    W = 1024
    P, Nn = S.camera_space(sc)
    Nb = torch.where(Nn[..., 2:] > 0, -Nn, Nn)
    p, nb, sd = P.numpy()[0], Nb.numpy()[0], sc["stddevs"].numpy()[0]
    prec = 0.01
    h = oracle.view_bandwidth(W, W, sc["focal"], p, nb, sd, 0.0)
    t = oracle.Tree(W, W, sc["focal"], p, h, oracle.cull_radius(h, prec), prec)
    e = t.export()
    n = t.n
    deg = e["degree"].copy()
    deg[n - 1:] = 0
    left, right, cnt, box = e["left"], e["right"], e["count"], e["box"]
    trunc = np.sqrt(-2.0 * h * h * np.log(prec / np.maximum(cnt, 1).astype(np.float64)))
    r_leaf = float(trunc[n - 1])

    def frontier(qx, qy):
        out, st = [], [0]
        while st:
            v = st.pop()
            if deg[v] >= 0:
                out.append(v)
                continue
            b = box[v]
            cx, cy = min(max(qx, b[0]), b[2]), min(max(qy, b[1]), b[3])
            if (qx - cx) ** 2 + (qy - cy) ** 2 < trunc[v] ** 2:
                st.append(right[v])
                st.append(left[v])
        return out

    rng = np.random.default_rng(0)
    leaf = rng.integers(0, n, args.pixels * 4)
    xy = e["leafxy"][leaf]
    nodes = []
    for qx, qy in np.round(xy):
        f = frontier(float(qx), float(qy))
        if f:
            nodes.append(f)
        if len(nodes) == args.pixels:
            break
    print(f"h = {h:.4f} px, leaf truncation radius {r_leaf:.2f} px, {len(nodes)} pixels on the surface")
    herm = np.mean([sum((deg[v] + 1) ** 2 for v in f) for f in nodes])
    print(f"Hermite evaluation now: {np.mean([len(f) for f in nodes]):.1f} nodes, {herm:.0f} series terms per pixel")
    print("| cell | Taylor degree q for 1e-4 | per-pixel Taylor terms | per-pixel conversion (shared by s^2) | total vs Hermite |")
    print("|---|---|---|---|---|")
    for s in (1, 2, 4):
        a_max = (s / 2.0 + r_leaf) / (math.sqrt(2.0) * h)
        q = taylor_degree(s, a_max, h=h)
        tay = np.mean([len(f) * (q + 1) ** 2 for f in nodes])
        conv = np.mean([sum((deg[v] + 1) * (q + 1) * (deg[v] + q + 2) for v in f) for f in nodes]) / (s * s)
        print(f"| {s}x{s} | {q} | {tay:.0f} | {conv:.0f} | {(tay + conv) / herm:.2f}x |")


if __name__ == "__main__":
    main()
