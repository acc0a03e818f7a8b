"""The calibration harness (procell/calibrate.py).

CPU: the searches' host logic on a stand-in problem whose expected counts are an analytic
Gaussian mixture with an exact Jacobian: the Gauss-Newton system's chain rule from (ratio,
mean, sd) to the unconstrained coordinates against torch autograd, Levenberg-Marquardt recovering the
parameters of a noise-free target, the particle swarm staying in its box and improving.
GPU: Levenberg-Marquardt on the smoothed form of the real calibration input reaches the
loss of the hidden parameters' neighbourhood within a few Jacobian passes.
"""
import math

import numpy as np
import pytest

torch = pytest.importorskip("torch")

from procell import calibrate as cb  # noqa: E402


class MixtureSmooth:
    """E_v = sum_k ratio_k A exp(-(x_v - mean_k)^2 / (2 sd_k^2)) and its exact Jacobian."""

    def __init__(self, n_values=60, amplitude=500.0):
        self.x = torch.linspace(0.0, 150.0, n_values, dtype=torch.float64)
        self.A = amplitude
        self.n_values = n_values

    def forward(self, prm):
        r, m, s = prm[..., 0][:, None, :], prm[..., 1][:, None, :], prm[..., 2][:, None, :]
        g = self.A * torch.exp(-(self.x[None, :, None] - m) ** 2 / (2 * s * s))
        return (r * g).sum(-1)

    def jacobian(self, prm):
        r, m, s = prm[..., 0][:, None, :], prm[..., 1][:, None, :], prm[..., 2][:, None, :]
        d = self.x[None, :, None] - m
        g = self.A * torch.exp(-d * d / (2 * s * s))
        J = torch.stack([g, r * g * d / (s * s), r * g * d * d / (s * s * s)], dim=-1)
        return (r * g).sum(-1), J

    def gauss_newton(self, prm, target):
        """The same contract as procell.smooth.Smooth.gauss_newton."""
        E, J = self.jacobian(prm)
        J = J.reshape(J.shape[0], J.shape[1], -1) / (1.0 + E)[..., None]
        r = torch.log1p(E) - torch.log1p(target)
        return (r * r).sum(1), J.transpose(1, 2) @ J, (J * r[..., None]).sum(1)


class MixtureProblem(cb.Problem):
    def __init__(self, hidden):
        self.n_types = len(hidden)
        self.smooth = MixtureSmooth()
        self.target = self.smooth.forward(torch.tensor([hidden], dtype=torch.float64))[0]

    def box(self):
        lo = torch.tensor([-3.0, math.log(cb.MEAN_RANGE[0]), math.log(cb.CV_RANGE[0])], dtype=torch.float64)
        hi = torch.tensor([3.0, math.log(cb.MEAN_RANGE[1]), math.log(cb.CV_RANGE[1])], dtype=torch.float64)
        return lo, hi

    def start(self, n, seed):
        g = torch.Generator().manual_seed(seed)
        lo, hi = self.box()
        return lo + torch.rand(n, self.n_types, 3, generator=g, dtype=torch.float64) * (hi - lo)

    def loss(self, theta):
        E = self.smooth.forward(self.params(theta))
        return ((torch.log1p(E) - torch.log1p(self.target)) ** 2).sum(dim=1)


HIDDEN = [(0.5, 40.0, 6.0), (0.3, 75.0, 9.0), (0.2, 110.0, 15.0)]


def test_gauss_newton_system_chain_rule():
    """Loss, J^T J and J^T r in theta against torch autograd of the residuals."""
    prob = MixtureProblem(HIDDEN)
    th = prob.start(4, 1)
    f, A, g = cb.gauss_newton_system(prob, th)

    def res(t):
        E = prob.smooth.forward(prob.params(t[None]))[0]
        return torch.log1p(E) - torch.log1p(prob.target)

    for c in range(th.shape[0]):
        J = torch.autograd.functional.jacobian(res, th[c]).reshape(prob.smooth.n_values, -1)
        r = res(th[c])
        assert torch.allclose(f[c], (r * r).sum())
        assert torch.allclose(A[c], J.T @ J, rtol=1e-9, atol=1e-12 * float((J.T @ J).abs().max()))
        assert torch.allclose(g[c], J.T @ r, rtol=1e-9, atol=1e-12 * float((J.T @ r).abs().max()))


def test_levenberg_marquardt_recovers_parameters():
    prob = MixtureProblem(HIDDEN)
    th0 = prob.start(32, 3)
    trace, snaps = cb.levenberg_marquardt(prob, th0, iters=60)
    assert trace[-1][1] < 1e-8 * trace[0][1]
    best = prob.params(snaps[-1][1][None])[0].numpy()
    best = best[np.argsort(best[:, 1])]  # types are exchangeable: order by mean
    assert np.allclose(best, np.array(HIDDEN), rtol=1e-4)
    losses = [l for _, l in trace]
    assert all(b <= a for a, b in zip(losses, losses[1:]))


def test_particle_swarm_stays_in_box_and_improves():
    prob = MixtureProblem(HIDDEN)
    th0 = prob.start(64, 5)
    trace, snaps = cb.particle_swarm(prob, th0, iters=40)
    lo, hi = prob.box()
    for _, th in snaps:
        assert torch.all(th >= lo) and torch.all(th <= hi)
    assert trace[-1][1] < 0.5 * trace[0][1]
    assert cb.first_below(trace, trace[-1][1]) is not None


@pytest.mark.gpu
def test_levenberg_marquardt_on_smoothed_form(engine):
    prob = cb.Problem(engine, seed=7)
    th0 = prob.start(64, 7)
    trace, snaps = cb.levenberg_marquardt(prob, th0, iters=12)
    with torch.no_grad():
        h = torch.tensor(prob.hidden, dtype=torch.float64, device="cuda")
        th_h = torch.stack([torch.log(h[:, 0]), torch.log(h[:, 1]), torch.log(h[:, 2] / h[:, 1])], dim=-1)[None]
        at_hidden = float(prob.loss(th_h)[0])
    prob.smooth.sync()
    # from uniform random starts to within 30% of the hidden parameters' own loss
    assert trace[-1][1] <= 1.3 * at_hidden, (trace[-1][1], at_hidden)


@pytest.mark.gpu
def test_plain_loss_matches_single_runs(engine):
    """The particle search's plain-simulator loss (all candidates as one batch, instance
    table reused between calls) equals the loss of each candidate's own pc_simulate."""
    prob = cb.Problem(engine, seed=7)
    th = prob.start(5, 3)
    L1 = prob.loss_plain(th).cpu().numpy()
    L2 = prob.loss_plain(th).cpu().numpy()
    L3 = prob.loss_plain(prob.start(5, 4)).cpu().numpy()
    P = prob.params(th).cpu().numpy()
    tgt = np.log1p(prob.target_np)
    for i in range(5):
        r = engine.simulate(prob.bins, [tuple(x) for x in P[i]], prob.t_max, prob.phi, prob.plain_seed)
        ref = ((np.log1p(r.totals.astype(np.float64)) - tgt) ** 2).sum()
        assert L1[i] == pytest.approx(ref, rel=1e-12)
    assert np.array_equal(L1, L2) and not np.array_equal(L1, L3)


@pytest.mark.gpu
def test_levenberg_marquardt_graph_equals_eager(engine):
    """The CUDA-graph replay of a Levenberg-Marquardt iteration computes exactly what the
    eager iteration computes."""
    prob = cb.Problem(engine, seed=7)
    th0 = prob.start(48, 11)
    ta, sa = cb.levenberg_marquardt(prob, th0, iters=6, graph=True)
    tb, sb = cb.levenberg_marquardt(prob, th0, iters=6, graph=False)
    assert [l for _, l in ta] == [l for _, l in tb]
    assert torch.equal(sa[-1][1], sb[-1][1])
