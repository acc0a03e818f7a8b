"""Calibration harness: recover cell-type parameters from an output histogram.

A target histogram is produced by the plain (stochastic, exact) form at hidden parameters
drawn from a seed. Candidates are scored with the smoothed form, loss
    L = sum_v (log(1 + E_v) - log(1 + C_v))^2
(E expected counts of the candidate, C the target counts), and searched two ways from the
same random starting population:
  * gradient descent: Adam on unconstrained coordinates, gradients from the smoothed
    form's adjoint kernel through procell.smooth.expected_counts (torch.autograd);
  * particle swarm: the same population as particles, forward passes only.
Both track the best loss over the population against wall time.

    python -m procell.calibrate [--candidates 256] [--seed 7]
"""
from __future__ import annotations

import argparse
import json
import math
import time

import numpy as np
import torch

from .smooth import Smooth, expected_counts

MEAN_RANGE = (20.0, 120.0)
CV_RANGE = (0.05, 0.5)  # sd / mean


class Problem:
    def __init__(self, engine, seed=7, n_bins=256, cells=100_000, n_types=3, t_max=168.0, h=0.5, paths=2):
        rng = np.random.default_rng(seed)
        v = np.exp(rng.uniform(0.0, math.log(1e4), n_bins))
        f = rng.multinomial(cells, np.full(n_bins, 1.0 / n_bins))
        self.bins = [(float(a), int(b)) for a, b in zip(v, f)]
        self.phi = float(min(a for a, b in self.bins if b > 0))
        ratios = rng.dirichlet(np.ones(n_types))
        ratios = ratios / ratios.sum()
        means = rng.uniform(30.0, 90.0, n_types)
        cvs = rng.uniform(0.1, 0.3, n_types)
        self.hidden = [(float(r), float(m), float(c * m)) for r, m, c in zip(ratios, means, cvs)]
        self.n_types, self.t_max = n_types, t_max
        res = engine.simulate(self.bins, self.hidden, t_max, self.phi, seed + 1000)
        self.smooth = Smooth(engine, self.bins, n_types, t_max, self.phi, h=h, paths=paths, seed=seed + 2000)
        assert np.array_equal(res.values, self.smooth.values)
        self.target = torch.tensor(res.totals.astype(np.float64), device="cuda")

    def params(self, theta):
        """theta [C, K, 3] = (ratio logit, log mean, log cv) -> (ratio, mean, sd)."""
        r = torch.softmax(theta[..., 0], dim=1)
        m = torch.exp(theta[..., 1])
        sd = m * torch.exp(theta[..., 2])
        return torch.stack([r, m, sd], dim=-1)

    def loss(self, theta):
        E = expected_counts(self.smooth, self.params(theta))
        return ((torch.log1p(E) - torch.log1p(self.target)) ** 2).sum(dim=1)

    def box(self):
        lo = torch.tensor([-3.0, math.log(MEAN_RANGE[0]), math.log(CV_RANGE[0])], dtype=torch.float64, device="cuda")
        hi = torch.tensor([3.0, math.log(MEAN_RANGE[1]), math.log(CV_RANGE[1])], dtype=torch.float64, device="cuda")
        return lo, hi

    def start(self, n, seed):
        g = torch.Generator(device="cuda").manual_seed(seed)
        lo, hi = self.box()
        u = torch.rand(n, self.n_types, 3, generator=g, dtype=torch.float64, device="cuda")
        return lo + u * (hi - lo)


def gradient_descent(prob, theta0, iters=150, lr=0.05, time_limit=None):
    theta = theta0.clone().requires_grad_(True)
    opt = torch.optim.Adam([theta], lr=lr)
    trace, best = [], float("inf")
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for it in range(iters):
        opt.zero_grad(set_to_none=True)
        L = prob.loss(theta)
        L.sum().backward()
        best = min(best, float(L.detach().min()))
        opt.step()
        trace.append((time.perf_counter() - t0, best))
        if time_limit and trace[-1][0] > time_limit:
            break
    return trace, theta.detach()


def particle_swarm(prob, theta0, iters=150, w=0.72, c1=1.49, c2=1.49, seed=1, time_limit=None):
    g = torch.Generator(device="cuda").manual_seed(seed)
    lo, hi = prob.box()
    x = theta0.clone()
    vel = torch.zeros_like(x)
    with torch.no_grad():
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        fx = prob.loss(x)
        pbest, pf = x.clone(), fx.clone()
        gi = int(torch.argmin(pf))
        gbest, gf = pbest[gi].clone(), float(pf[gi])
        trace = [(time.perf_counter() - t0, gf)]
        for it in range(iters):
            r1 = torch.rand(x.shape, generator=g, dtype=x.dtype, device=x.device)
            r2 = torch.rand(x.shape, generator=g, dtype=x.dtype, device=x.device)
            vel = w * vel + c1 * r1 * (pbest - x) + c2 * r2 * (gbest - x)
            x = torch.minimum(torch.maximum(x + vel, lo), hi)
            fx = prob.loss(x)
            better = fx < pf
            pbest[better] = x[better]
            pf = torch.where(better, fx, pf)
            gi = int(torch.argmin(pf))
            if float(pf[gi]) < gf:
                gf, gbest = float(pf[gi]), pbest[gi].clone()
            trace.append((time.perf_counter() - t0, gf))
            if time_limit and trace[-1][0] > time_limit:
                break
    return trace, gbest


def time_to(trace, level):
    for t, l in trace:
        if l <= level:
            return t
    return None


def compare(engine, candidates=256, seed=7, gd_iters=150, pso_iters=300):
    prob = Problem(engine, seed=seed)
    theta0 = prob.start(candidates, seed)
    prob.loss(theta0)  # warm-up (allocations, first launches)
    gd, th_gd = gradient_descent(prob, theta0, iters=gd_iters)
    ps, th_ps = particle_swarm(prob, theta0, iters=pso_iters)
    level = max(ps[-1][1], gd[-1][1])  # the loss both searches reach
    t_gd, t_ps = time_to(gd, level), time_to(ps, level)
    return {
        "candidates": candidates,
        "hidden": prob.hidden,
        "gd": {"iters": len(gd), "seconds": gd[-1][0], "best_loss": gd[-1][1]},
        "pso": {"iters": len(ps) - 1, "seconds": ps[-1][0], "best_loss": ps[-1][1]},
        "equal_loss": level,
        "gd_seconds_to_equal_loss": t_gd,
        "pso_seconds_to_equal_loss": t_ps,
        "speedup": (t_ps / t_gd) if (t_gd and t_ps) else None,
    }


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--candidates", type=int, default=256)
    ap.add_argument("--seed", type=int, default=7)
    ap.add_argument("--gd-iters", type=int, default=150)
    ap.add_argument("--pso-iters", type=int, default=300)
    a = ap.parse_args()
    from . import Engine
    eng = Engine(0)
    print(json.dumps(compare(eng, a.candidates, a.seed, a.gd_iters, a.pso_iters)))


if __name__ == "__main__":
    main()
