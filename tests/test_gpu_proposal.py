"""Learned proposal (tensor-core network) for the stochastic sampling mode:
its training rows, unbiasedness of the weighted estimator against FP64 exact
Gaussian mixtures, and what training gains over an untrained network."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu
DEV = "cuda:0"


@pytest.fixture(scope="module")
def setup():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from unbiased_differentiable_splatting_gb300 import _lib, proposal, scenes
    from unbiased_differentiable_splatting_gb300.cudaExtensions import sampling
    _lib.load()
    sc = scenes.harmonic_scene(n=6000, sd_range=(0.01, 0.02), width=48, seed=4)
    P, Nn = scenes.camera_space(sc)
    P = P.to(DEV)
    Nn = torch.where(Nn[..., 2:] > 0, -Nn, Nn).contiguous().to(DEV)
    sd = sc["stddevs"].to(DEV)
    args = (48, 48, sc["focal"], P, Nn, sd)
    net = proposal.ProposalNet(DEV, seed=1)
    X, t = proposal.dataset(*args, 0.0, 1e-4, stride=2, draws=8, seed=3)
    losses = net.train(X, t, steps=400, batch=16384, lr=3e-3).cpu()
    assert not net.failed()
    return dict(proposal=proposal, sampling=sampling, args=args, net=net, X=X, t=t, losses=losses, sc=sc)


def exact_mixture(setup, values):
    """FP64 sum_j G_j(x) f_j / sum_j G_j(x) over the visible splats."""
    sampling = setup["sampling"]
    W, H, f, P, Nn, sd = setup["args"]
    tree = sampling.build_tree(W, H, f, P, Nn, sd, 8, 0.0, 1e-4)
    n = tree["n_visible"]
    h = tree["h"]
    xy = tree["centre"][n - 1:].double()  # leaf screen positions
    ids = tree["ids"].long()
    gi, gj = torch.meshgrid(torch.arange(W, dtype=torch.float64), torch.arange(H, dtype=torch.float64),
                            indexing="ij")
    d2 = (gi[..., None] - xy[:, 0]) ** 2 + (gj[..., None] - xy[:, 1]) ** 2
    G = torch.exp(-d2 / (2 * h * h))
    fv = values[0, ids].double()  # (n, C)
    mass = G.sum(-1)
    return (G @ fv) / mass[..., None], mass


def test_training_rows_and_loss(setup):
    X, t, losses = setup["X"], setup["t"], setup["losses"]
    assert X.shape[0] > 10000 and X.shape[1] == 16
    assert float(t.min()) >= 0.0 and float(t.max()) <= 1.0
    assert torch.isfinite(X).all()
    assert float(losses[-20:].mean()) < float(losses[:5].mean())
    # the network's probabilities track the exact branch probabilities
    q = torch.softmax(setup["net"].logits(X[:50000]), -1)[:, 0]
    err = float((q - t[:50000]).abs().mean())
    base = float((t[:50000] - t[:50000].mean()).abs().mean())
    assert err < 0.6 * base, (err, base)


@pytest.mark.parametrize("learned", [False, True])
def test_weighted_estimator_unbiased(setup, learned):
    """Mean of the weighted estimate over many seeds against the FP64 exact
    mixture of the splat values (within the Monte-Carlo error and the FGT
    truncation precision)."""
    proposal = setup["proposal"]
    g = torch.Generator().manual_seed(5)
    values = torch.rand(1, setup["args"][3].shape[1], 2, generator=g).to(DEV)
    exact, mass = exact_mixture(setup, values.cpu())
    acc, acc2, S = 0, 0, 60
    fb = 0
    for s in range(S):
        idx, w, fbm, nfb = proposal.sample(*setup["args"], 8, 0.0, 1e-4, net=setup["net"] if learned else None,
                                           ess_tau=0.3, seed=1000 + s)
        e = proposal.estimate(idx, w, values)[0].double().cpu()
        acc = acc + e
        acc2 = acc2 + e * e
        fb += int(nfb.sum())
    mean = acc / S
    var = (acc2 / S - mean ** 2).clamp_min(0)
    se = (var / S).sqrt()
    live = mass > 1e-2
    z = ((mean - exact).abs() / (se + 1e-3 * exact.abs() + 1e-6))[live]
    # training is deterministic (fixed row order, gradients summed in block
    # order), so these figures are the same on every run; a bias would raise
    # z over many pixels
    print("z mean / q995 / max", float(z.mean()), float(torch.quantile(z, 0.995)), float(z.max()))
    assert float(z.mean()) < 1.5, float(z.mean())
    assert float(torch.quantile(z, 0.995)) < 4.5, float(torch.quantile(z, 0.995))
    assert float(z.max()) < 6.0, float(z.max())


def test_training_is_deterministic(setup):
    """The same data and seeds give the same rows and the same trained
    parameters, bit for bit."""
    proposal = setup["proposal"]
    X2, t2 = proposal.dataset(*setup["args"], 0.0, 1e-4, stride=2, draws=8, seed=3)
    assert torch.equal(X2, setup["X"]) and torch.equal(t2, setup["t"])
    net2 = proposal.ProposalNet(DEV, seed=1)
    losses = net2.train(X2, t2, steps=400, batch=16384, lr=3e-3).cpu()
    assert torch.equal(net2.params, setup["net"].params)
    assert torch.equal(losses, setup["losses"])


def test_trained_network_gains(setup):
    """Estimator variance with the trained network against the same network
    untrained; both unbiased, training lowers the variance and the fallbacks."""
    proposal = setup["proposal"]
    g = torch.Generator().manual_seed(6)
    values = torch.rand(1, setup["args"][3].shape[1], 1, generator=g).to(DEV)
    _, mass = exact_mixture(setup, values.cpu())
    live = (mass > 1e-2).to(DEV)
    untrained = proposal.ProposalNet(DEV, seed=1)

    def stats(net):
        es, nf = [], 0
        for s in range(24):
            idx, w, fbm, nfb = proposal.sample(*setup["args"], 8, 0.0, 1e-4, net=net, ess_tau=0.0, seed=2000 + s)
            es.append(proposal.estimate(idx, w, values)[0, ..., 0])
        e = torch.stack(es)
        return float(e.var(0)[live].mean())

    v_trained, v_untrained = stats(setup["net"]), stats(untrained)
    print("estimator variance: trained", v_trained, "untrained", v_untrained)
    assert v_trained < 0.5 * v_untrained, (v_trained, v_untrained)
