"""Discrete adjoint on the GPU against FP64 forward sensitivities and central
finite differences of the same frozen step sequence (oracle/sensitivity.py).

Workload shape of the differentiation config: a 256-species x 256-reaction
network with k = 10^U(-3,3); targets from perturbed rate constants
k * exp(N(0, 0.3^2)); here on a shortened horizon (t in [0,1], 9 samples)
so that the CPU checks finish in seconds.
"""
import numpy as np
import pytest

from lassie_gb300 import synth
from lassie_gb300.adjoint import adjoint_batch, trajectory_misfit
from oracle import oracle as O
from oracle import sensitivity as S

pytestmark = pytest.mark.gpu


def problem(copy=0, t_end=1.0, n=9):
    base, k_t = synth.make_c5(copy + 1)
    m = synth.shorten(base[copy], t_end, n)
    mt = synth.shorten(base[copy], t_end, n)
    mt.k = k_t[copy]
    target, _, rc = O.solve(mt)
    assert rc == 0
    return m, target


def test_adjoint_matches_forward_sensitivities(gpu):
    m, target = problem()
    out_o, st_o, rc, kinds, dts, samp = O.solve_recorded(m)
    loss, gk, gx, outs, stats = adjoint_batch([m], [target], root="sqrt", deadline_s=120,
                                              engine="fp64")
    g = gk[0]
    assert stats[0]["status"] == 0
    # the FP64 GPU forward took the oracle's step sequence
    assert stats[0]["be_steps"] == int(np.sum(kinds >= 1))
    assert stats[0]["rkf_accepts"] == int(np.sum(kinds == 0))
    assert loss[0] == pytest.approx(float(np.sum((out_o - target) ** 2)), rel=1e-9)
    logk = np.log(m.k)
    rng = np.random.default_rng(11)
    for _ in range(2):
        v = rng.normal(size=m.n_reactions)
        tl = S.tlm_directional(m, logk, target, kinds, dts, samp, v)
        ad = float(g @ v)
        assert abs(ad - tl) <= 1e-4 * np.abs(g).sum() * np.abs(v).max(), (ad, tl)


def test_adjoint_matches_central_differences(gpu):
    m, target = problem()
    _, _, _, kinds, dts, samp = O.solve_recorded(m)
    _, gk, _, _, _ = adjoint_batch([m], [target], root="sqrt", deadline_s=120, engine="fp64")
    g = gk[0]
    idx = list(np.argsort(-np.abs(g))[:3])  # the three most sensitive constants
    fd = S.fd_gradient(m, np.log(m.k), target, kinds, dts, samp, idx, h=1e-6)
    assert np.allclose(g[idx], fd, rtol=1e-4, atol=1e-6 * np.abs(g).max())


def test_mixed_forward_gives_the_fp64_gradient(gpu):
    """The mixed forward (FP32 LU + FP64 refinement) records the same step
    sequence on this case (t in [0, 0.8]: backward-Euler steps only, and
    insensitive to last-bit differences of the linear solve); its gradient
    then agrees with the FP64 forward's."""
    m, target = problem(t_end=0.8, n=9)
    l64, g64, _, _, s64 = adjoint_batch([m], [target], root="sqrt", engine="fp64")
    lmx, gmx, _, _, smx = adjoint_batch([m], [target], root="sqrt", engine="mixed")
    assert (smx[0]["be_steps"], smx[0]["rkf_accepts"]) == (s64[0]["be_steps"], s64[0]["rkf_accepts"])
    assert lmx[0] == pytest.approx(l64[0], rel=1e-6)
    assert np.abs(gmx[0] - g64[0]).max() <= 1e-6 * np.abs(g64[0]).sum()


def test_checkpoint_interval_does_not_change_the_gradient(gpu):
    m, target = problem()
    ref = adjoint_batch([m], [target], ckpt_every=1, root="sqrt")[1][0]
    for K in (2, 8, 64):
        g = adjoint_batch([m], [target], ckpt_every=K, root="sqrt")[1][0]
        assert np.array_equal(g, ref), K


def test_batch_gradients_are_independent(gpu):
    pairs = [problem(c) for c in range(3)]
    models = [p[0] for p in pairs]
    targets = [p[1] for p in pairs]
    loss, gk, _, _, _ = adjoint_batch(models, targets, root="sqrt")
    for q in range(3):
        l1, g1, _, _, _ = adjoint_batch([models[q]], [targets[q]], root="sqrt")
        assert loss[q] == l1[0]
        assert np.array_equal(gk[q], g1[0])


def test_torch_autograd(gpu):
    torch = pytest.importorskip("torch")
    pairs = [problem(c) for c in range(2)]
    models = [p[0] for p in pairs]
    targets = [p[1] for p in pairs]
    logk = torch.tensor(np.log(np.stack([m.k for m in models])), dtype=torch.float64,
                        requires_grad=True)
    L = trajectory_misfit(logk, models, targets)
    (L[0] + 2.0 * L[1]).backward()
    # the same rate constants the autograd path used: exp(log k)
    for b, m in enumerate(models):
        m.k = np.exp(logk.detach().numpy()[b])
    _, gk, _, _, _ = adjoint_batch(models, targets)
    assert np.allclose(logk.grad.numpy(), np.stack([gk[0], 2.0 * gk[1]]), rtol=1e-12, atol=0)


def test_fit_rate_constants_reduces_the_misfit(gpu):
    """The parameter-fit loop: from rate constants perturbed by exp(N(0, 0.3^2))
    towards the ones that made the targets, Adam on the adjoint gradient
    lowers the misfit, at least halving it within 30 iterations."""
    from lassie_gb300.adjoint import fit_rate_constants
    base, k_t = synth.make_c5(2)
    models, targets = [], []
    for q in range(2):
        m = synth.shorten(base[q], 0.8, 9)
        mt = synth.shorten(base[q], 0.8, 9)
        mt.k = k_t[q]
        tgt, _, rc = O.solve(mt)
        assert rc == 0
        models.append(m)
        targets.append(tgt)
    log_k, hist = fit_rate_constants(models, targets, iters=30, lr=0.05)
    assert np.all(np.isfinite(hist))
    assert min(hist) < 0.5 * hist[0] and hist[-1] < hist[0], (hist[0], min(hist), hist[-1])
