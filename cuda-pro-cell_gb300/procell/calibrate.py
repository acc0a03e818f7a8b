"""Calibration harness: recover cell-type parameters from an output histogram.

A target histogram is produced by the plain (stochastic, exact) form at hidden parameters
drawn from a seed. Candidates are scored by
    L = sum_v (log(1 + E_v) - log(1 + C_v))^2
(E the candidate's counts, C the target counts), and searched three ways from the same
random starting population:
  * gradient descent on the smoothed form: Adam on unconstrained coordinates, gradients
    from the smoothed form's adjoint kernel through procell.smooth.expected_counts;
  * a particle swarm on the smoothed form (forward passes only);
  * a particle swarm on the plain simulator itself: every iteration runs all candidates as
    the instances of one batch (pc_simulate_batch), the search a practitioner without a
    differentiable model would run.
Each search keeps its best parameters over time; afterwards every snapshot is scored with
one accurate common loss (the smoothed form with many lineages per cell, another seed), so
the searches are compared on the same scale.

    python -m procell.calibrate [--candidates 256] [--seed 7] [--gd-iters 300] [--pso-seconds 40]
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


def problem_inputs(seed=7, n_bins=256, cells=100_000, n_types=3):
    """The calibration input: 256 bins (fluorescence log-uniform on [1, 1e4], 1e5 cells spread
    uniformly), phi = the smallest value, and hidden parameters drawn from the seed (Dirichlet
    ratios, means U[30, 90], sd = U[0.1, 0.3] x mean)."""
    rng = np.random.default_rng(seed)
    v = np.exp(rng.uniform(0.0, math.log(1e4), n_bins))
    f = rng.multinomial(cells, np.full(n_bins, 1.0 / n_bins))
    bins = [(float(a), int(b)) for a, b in zip(v, f)]
    phi = float(min(a for a, b in bins if b > 0))
    ratios = rng.dirichlet(np.ones(n_types))
    ratios = ratios / ratios.sum()
    means = rng.uniform(30.0, 90.0, n_types)
    cvs = rng.uniform(0.1, 0.3, n_types)
    hidden = [(float(r), float(m), float(c * m)) for r, m, c in zip(ratios, means, cvs)]
    return bins, phi, hidden


class Problem:
    def __init__(self, engine, seed=7, n_bins=256, cells=100_000, n_types=3, t_max=168.0, h=0.5, paths=2):
        self.bins, self.phi, self.hidden = problem_inputs(seed, n_bins, cells, n_types)
        self.n_types, self.t_max = n_types, t_max
        res = engine.simulate(self.bins, self.hidden, t_max, self.phi, seed + 1000)
        self.smooth_h, self.smooth_paths, self.smooth_seed = h, paths, seed + 2000
        self.smooth = Smooth(engine, self.bins, n_types, t_max, self.phi, h=h, paths=paths, seed=seed + 2000)
        assert np.array_equal(res.values, self.smooth.values)
        self.engine = engine
        self.target_np = res.totals.astype(np.float64)
        self.target = torch.tensor(self.target_np, device="cuda")
        self.plain_seed = seed + 3000
        from . import _lib
        self._bins_np = _lib.bins_numpy(self.bins)
        self._accurate = None

    def loss_accurate(self, theta, paths=32):
        """The common yardstick: the smoothed form with many lineages per cell (another
        seed), i.e. close to the plain model's expectation."""
        if self._accurate is None:
            self._accurate = Smooth(self.engine, self.bins, self.n_types, self.t_max, self.phi, h=self.smooth_h,
                                    paths=paths, seed=self.smooth_seed + 5000)
        with torch.no_grad():
            out = []
            for chunk in torch.split(theta, 256):
                E = self._accurate.forward(self.params(chunk))
                out.append(((torch.log1p(E) - torch.log1p(self.target)) ** 2).sum(dim=1))
            return torch.cat(out)

    def params(self, theta):
        """theta [C, K, 3] = (ratio logit, log mean, log cv) -> (ratio, mean, sd)."""
        r = torch.softmax(theta[..., 0], dim=1)
        m = torch.exp(theta[..., 1])
        sd = m * torch.exp(theta[..., 2])
        return torch.stack([r, m, sd], dim=-1)

    def loss(self, theta):
        E = expected_counts(self.smooth, self.params(theta))
        return ((torch.log1p(E) - torch.log1p(self.target)) ** 2).sum(dim=1)

    def loss_plain(self, theta, seed=None):
        """Loss of every candidate under the plain simulator: the candidates run as the
        instances of one batch (one seed for all: common random numbers)."""
        import ctypes
        from . import _lib
        P = self.params(theta).detach().cpu().numpy()
        seed = self.plain_seed if seed is None else seed
        n = P.shape[0]
        keep = [self._bins_np]
        arr = (_lib.Instance * n)()
        for i in range(n):
            t = _lib.types_numpy([tuple(row) for row in P[i]])
            keep.append(t)
            arr[i].bins = self._bins_np.ctypes.data_as(ctypes.POINTER(_lib.Bin))
            arr[i].n_bins = len(self._bins_np)
            arr[i].types = t.ctypes.data_as(ctypes.POINTER(_lib.CellType))
            arr[i].n_types = len(t)
            arr[i].t_max, arr[i].phi, arr[i].seed = self.t_max, self.phi, seed
        hs = (_lib.Histogram * n)()
        eng = self.engine
        eng._check(eng.L.pc_simulate_batch(eng.ctx, arr, n, hs))
        tgt = np.log1p(self.target_np)
        out = np.empty(n)
        for i in range(n):
            h = hs[i]
            tot = np.ctypeslib.as_array(h.totals, shape=(int(h.n_values),)).astype(np.float64)
            out[i] = ((np.log1p(tot) - tgt) ** 2).sum()
            eng.L.pc_histogram_free(ctypes.byref(h))
        return torch.tensor(out, dtype=torch.float64, device=theta.device)

    def box(self):
        lo = torch.tensor([-3.0, math.log(MEAN_RANGE[0]), math.log(CV_RANGE[0])], dtype=torch.float64, device="cuda")
        hi = torch.tensor([3.0, math.log(MEAN_RANGE[1]), math.log(CV_RANGE[1])], dtype=torch.float64, device="cuda")
        return lo, hi

    def start(self, n, seed):
        g = torch.Generator(device="cuda").manual_seed(seed)
        lo, hi = self.box()
        u = torch.rand(n, self.n_types, 3, generator=g, dtype=torch.float64, device="cuda")
        return lo + u * (hi - lo)


def gradient_descent(prob, theta0, iters=150, lr=0.1, lr_end=0.002, time_limit=None):
    """Adam from every candidate at once, learning rate decaying from lr to lr_end (cosine)."""
    theta = theta0.clone().requires_grad_(True)
    opt = torch.optim.Adam([theta], lr=lr)
    trace, best = [], float("inf")
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    snaps = []
    for it in range(iters):
        for group in opt.param_groups:
            group["lr"] = lr_end + 0.5 * (lr - lr_end) * (1.0 + math.cos(math.pi * it / max(1, iters - 1)))
        opt.zero_grad(set_to_none=True)
        L = prob.loss(theta)
        L.sum().backward()
        i = int(torch.argmin(L.detach()))
        if float(L[i]) < best:
            best = float(L[i])
            snaps.append((time.perf_counter() - t0, theta.detach()[i].clone()))
        opt.step()
        trace.append((time.perf_counter() - t0, best))
        if time_limit and trace[-1][0] > time_limit:
            break
    return trace, snaps


def particle_swarm(prob, theta0, iters=150, w=0.7298, c1=1.49618, c2=1.49618, seed=1, time_limit=None,
                   loss=None):
    """Particle swarm with constriction coefficients and a ring neighbourhood (each particle
    follows the best of itself and its two neighbours), the standard choice for multimodal
    objectives; particles stay in the search box."""
    loss = loss or prob.loss
    g = torch.Generator(device="cuda").manual_seed(seed)
    lo, hi = prob.box()
    x = theta0.clone()
    vel = torch.zeros_like(x)
    vmax = 0.5 * (hi - lo)
    with torch.no_grad():
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        fx = loss(x)
        pbest, pf = x.clone(), fx.clone()
        gf = float(pf.min())
        trace = [(time.perf_counter() - t0, gf)]
        snaps = [(trace[0][0], pbest[int(torch.argmin(pf))].clone())]
        for it in range(iters):
            # best personal best among each particle's ring neighbourhood {i-1, i, i+1}
            cand = torch.stack([pf.roll(1), pf, pf.roll(-1)])
            j = cand.argmin(dim=0)
            nb = torch.where((j == 0)[:, None, None], pbest.roll(1, 0),
                             torch.where((j == 1)[:, None, None], pbest, pbest.roll(-1, 0)))
            r1 = torch.rand(x.shape, generator=g, dtype=x.dtype, device=x.device)
            r2 = torch.rand(x.shape, generator=g, dtype=x.dtype, device=x.device)
            vel = w * vel + c1 * r1 * (pbest - x) + c2 * r2 * (nb - x)
            vel = torch.minimum(torch.maximum(vel, -vmax), vmax)
            x = torch.minimum(torch.maximum(x + vel, lo), hi)
            fx = loss(x)
            better = fx < pf
            pbest[better] = x[better]
            pf = torch.where(better, fx, pf)
            gi = int(torch.argmin(pf))
            if float(pf[gi]) < gf:
                gf = float(pf[gi])
                snaps.append((time.perf_counter() - t0, pbest[gi].clone()))
            trace.append((time.perf_counter() - t0, gf))
            if time_limit and trace[-1][0] > time_limit:
                break
    return trace, snaps


def accurate_trace(prob, snaps):
    """(time, accurate loss of the search's best parameters so far) for each snapshot."""
    if not snaps:
        return []
    L = prob.loss_accurate(torch.stack([th for _, th in snaps])).cpu().numpy()
    return [(t, float(v)) for (t, _), v in zip(snaps, L)]


def first_below(trace, level):
    """First time a (time, loss) trace is at or below `level` (losses need not decrease)."""
    for t, l in trace:
        if l <= level:
            return t
    return None


def compare(engine, candidates=256, seed=7, gd_iters=300, pso_seconds=40.0, paths=2):
    """Gradient descent on the smoothed form against particle swarms (on the smoothed form
    and on the plain simulator through the batched form), all from one population, all
    scored afterwards with the same accurate loss. The headline level is the worse of the
    plain-simulator swarm's and gradient descent's final accurate losses (a level both
    reach); the ratio is the swarm's time to reach it over gradient descent's."""
    prob = Problem(engine, seed=seed, paths=paths)
    theta0 = prob.start(candidates, seed)
    gradient_descent(prob, theta0, iters=3)  # warm-up of every code path
    particle_swarm(prob, theta0, iters=3)
    particle_swarm(prob, theta0, iters=2, loss=prob.loss_plain)
    gd, gd_snaps = gradient_descent(prob, theta0, iters=gd_iters)
    ps, ps_snaps = particle_swarm(prob, theta0, iters=1_000_000, time_limit=pso_seconds)
    pp, pp_snaps = particle_swarm(prob, theta0, iters=1_000_000, time_limit=pso_seconds, loss=prob.loss_plain)
    acc_gd, acc_ps, acc_pp = (accurate_trace(prob, x) for x in (gd_snaps, ps_snaps, pp_snaps))
    with torch.no_grad():
        hidden = torch.tensor([prob.hidden], dtype=torch.float64, device="cuda")
        th_h = torch.stack([torch.log(hidden[0, :, 0]), torch.log(hidden[0, :, 1]),
                            torch.log(hidden[0, :, 2] / hidden[0, :, 1])], dim=-1)[None]
        l_true = float(prob.loss_accurate(th_h)[0])

    def best_final(tr):
        return min(l for _, l in tr)

    head = max(best_final(acc_pp), best_final(acc_gd))
    levels = sorted({head, 1.05 * head, 1.2 * head, 1.5 * head, l_true}, reverse=True)
    table = []
    for L in levels:
        tg, tp, ts = first_below(acc_gd, L), first_below(acc_pp, L), first_below(acc_ps, L)
        table.append({"accurate_loss": L, "gd_seconds": tg, "pso_plain_seconds": tp, "pso_smooth_seconds": ts,
                      "ratio_plain": (tp / tg) if (tg and tp) else None,
                      "ratio_smooth": (ts / tg) if (tg and ts) else None})
    tg, tp = first_below(acc_gd, head), first_below(acc_pp, head)
    return {
        "candidates": candidates,
        "lineages_per_cell": paths,
        "hidden": prob.hidden,
        "accurate_loss_at_hidden": l_true,
        "gd": {"iters": len(gd), "seconds": gd[-1][0], "best_smoothed_loss": gd[-1][1],
               "best_accurate_loss": best_final(acc_gd), "method": "Adam on the smoothed form, cosine lr 0.1 -> 0.002"},
        "pso_smooth": {"iters": len(ps) - 1, "seconds": ps[-1][0], "best_smoothed_loss": ps[-1][1],
                       "best_accurate_loss": best_final(acc_ps),
                       "method": "particle swarm on the smoothed form (constriction, ring neighbourhood)"},
        "pso_plain": {"iters": len(pp) - 1, "seconds": pp[-1][0], "best_plain_loss": pp[-1][1],
                      "best_accurate_loss": best_final(acc_pp),
                      "method": "particle swarm on the plain simulator, candidates as one pc_simulate_batch"},
        "equal_loss": head,
        "equal_loss_is": "accurate loss both gradient descent and the plain-simulator swarm reach",
        "gd_seconds_to_equal_loss": tg,
        "pso_seconds_to_equal_loss": tp,
        "speedup": (tp / tg) if (tg and tp) else None,
        "levels": table,
    }


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--candidates", type=int, default=256)
    ap.add_argument("--seed", type=int, default=7)
    ap.add_argument("--gd-iters", type=int, default=300)
    ap.add_argument("--pso-seconds", type=float, default=40.0)
    ap.add_argument("--paths", type=int, default=2)
    a = ap.parse_args()
    from . import Engine
    eng = Engine(0)
    print(json.dumps(compare(eng, a.candidates, a.seed, a.gd_iters, a.pso_seconds, a.paths)))


if __name__ == "__main__":
    main()
