"""Calibration harness: recover cell-type parameters from an output histogram.

A target histogram is produced by the plain (stochastic, exact) form at hidden parameters
drawn from a seed. Candidates are scored by
    L = sum_v (log(1 + E_v) - log(1 + C_v))^2
(E the candidate's counts, C the target counts), and searched four ways from the same
random starting population:
  * Levenberg-Marquardt on the smoothed form: the Gauss-Newton system (J^T J, J^T r, loss)
    from one pass of the forward-mode Jacobian kernel per iteration, reduced on the device
    (pc_smooth_gauss_newton);
  * gradient descent on the smoothed form: Adam on unconstrained coordinates, gradients
    from the smoothed form's adjoint kernel through procell.smooth.expected_counts;
  * a particle swarm on the smoothed form (forward passes only);
  * a particle swarm on the plain simulator itself: every iteration runs all candidates as
    the instances of one batch (prepared once; pc_batch_set_types, pc_batch_run,
    pc_batch_totals per iteration), the search a practitioner without a differentiable
    model would run.
Each search keeps its best parameters over time; afterwards every snapshot is scored with
one accurate common loss (the smoothed form with many lineages per cell, another seed), so
the searches are compared on the same scale, and with a model-neutral one: the plain
simulator's own loss averaged over independent seeds (no smoothing, and no random numbers
shared with any search).

    python -m procell.calibrate [--candidates 256] [--seed 7] [--lm-iters 40] [--gd-iters 300] [--pso-seconds 40]
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
        # log(1 + target) of the residuals r_v = log(1 + E_v) - log(1 + target_v), once (FP64
        # logarithms run on GB300's slow FP64 pipe)
        self.target_log = torch.log1p(self.target)
        self.plain_seed = seed + 3000
        self.neutral_seed = seed + 4000
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
                out.append(((torch.log1p(E) - self.target_log) ** 2).sum(dim=1))
            return torch.cat(out)

    def loss_plain_mean(self, theta, n_seeds=16, chunk=256):
        """The model-neutral yardstick: the plain simulator's loss of every candidate averaged
        over `n_seeds` independent seeds (seeds no search uses). Each chunk of candidates x
        seeds runs as the instances of one batch. Returns a numpy array [C]."""
        P = self.params(theta).detach().cpu().numpy()
        V = len(self.target_np)
        tgt = np.log1p(self.target_np)
        out = []
        for c0 in range(0, P.shape[0], chunk):
            Pc = P[c0:c0 + chunk]
            rows = [[tuple(float(x) for x in r) for r in Pc[i]] for i in range(len(Pc))]
            inst = [(self._bins_np, rows[i], self.t_max, self.phi, self.neutral_seed + 7919 * s)
                    for s in range(n_seeds) for i in range(len(Pc))]
            b = self.engine.batch(inst)
            try:
                b.run()
                off, tot = b.totals()
            finally:
                b.close()
            assert int(off[-1]) == n_seeds * len(Pc) * V
            C = tot.astype(np.float64).reshape(n_seeds, len(Pc), V)
            out.append(((np.log1p(C) - tgt) ** 2).sum(axis=2).mean(axis=0))
        return np.concatenate(out)

    def params(self, theta):
        """theta [C, K, 3] = (ratio logit, log mean, log cv) -> (ratio, mean, sd)."""
        r = torch.softmax(theta[..., 0], dim=1)
        m = torch.exp(theta[..., 1])
        sd = m * torch.exp(theta[..., 2])
        return torch.stack([r, m, sd], dim=-1)

    def loss(self, theta):
        E = expected_counts(self.smooth, self.params(theta))
        return ((torch.log1p(E) - self.target_log) ** 2).sum(dim=1)

    def loss_plain(self, theta, seed=None):
        """Loss of every candidate under the plain simulator: the candidates are the
        instances of one batch (one seed for all: common random numbers). The batch is
        prepared once (bins, value sets, device tables); each call only replaces the cell
        types (pc_batch_set_types), runs it and reads all merged totals at once
        (pc_batch_totals)."""
        from . import _lib
        P = self.params(theta).detach().cpu().numpy()
        seed = self.plain_seed if seed is None else int(seed)
        n, K = P.shape[0], P.shape[1]
        types = np.zeros(n * K, _lib.TYPE_DTYPE)
        types["ratio"], types["mean"], types["sd"] = P[..., 0].ravel(), P[..., 1].ravel(), P[..., 2].ravel()
        cache = getattr(self, "_plain_batch", None)
        if cache is None or cache[0] != (n, seed):
            if cache is not None:
                cache[1].close()
            rows = [[tuple(r) for r in P[i]] for i in range(n)]
            batch = self.engine.batch([(self._bins_np, rows[i], self.t_max, self.phi, seed) for i in range(n)])
            cache = self._plain_batch = ((n, seed), batch)
        else:
            cache[1].set_types(types)
        batch = cache[1]
        batch.run()
        off, tot = batch.totals()
        V = len(self.target_np)
        assert int(off[-1]) == n * V
        C = torch.from_numpy(tot.view(np.int64).reshape(n, V)).to(theta.device).to(torch.float64)
        return ((torch.log1p(C) - self.target_log) ** 2).sum(dim=1)

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
    """Adam from every candidate at once, learning rate decaying from lr to lr_end (cosine),
    each step projected onto the search box that every search shares."""
    lo, hi = prob.box()
    theta = theta0.clone().requires_grad_(True)
    opt = torch.optim.Adam([theta], lr=lr)
    trace, best = [], float("inf")
    if theta.is_cuda:
        torch.cuda.synchronize()
    t0 = time.perf_counter()
    snaps = []
    for it in range(iters):
        for group in opt.param_groups:
            group["lr"] = lr_end + 0.5 * (lr - lr_end) * (1.0 + math.cos(math.pi * it / max(1, iters - 1)))
        opt.zero_grad(set_to_none=True)
        L = prob.loss(theta)
        L.sum().backward()
        Ld = L.detach()
        i = int(torch.argmin(Ld))
        if float(Ld[i]) < best:
            best = float(Ld[i])
            snaps.append((time.perf_counter() - t0, theta.detach()[i].clone()))
        opt.step()
        with torch.no_grad():
            theta.copy_(torch.minimum(torch.maximum(theta, lo), hi))
        trace.append((time.perf_counter() - t0, best))
        if time_limit and trace[-1][0] > time_limit:
            break
    return trace, snaps


def param_jacobian(th, prm):
    """dP/dtheta [n, 3K, 3K] (index 3k + q on both sides) of prob.params: ratios = softmax of
    the logits, mean = e^b, sd = mean e^c."""
    n, K = th.shape[0], th.shape[1]
    r = torch.softmax(th[..., 0], dim=1)
    D = torch.zeros(n, K, 3, K, 3, dtype=th.dtype, device=th.device)
    D[:, :, 0, :, 0] = torch.diag_embed(r) - r[:, :, None] * r[:, None, :]
    k = torch.arange(K, device=th.device)
    D[:, k, 1, k, 1] = prm[..., 1]
    D[:, k, 2, k, 1] = prm[..., 2]
    D[:, k, 2, k, 2] = prm[..., 2]
    return D.reshape(n, 3 * K, 3 * K)


def gauss_newton_system(prob, th):
    """Loss [n], J^T J [n, 3K, 3K] and J^T r [n, 3K] of the residuals r_v = log(1 + E_v) -
    log(1 + C_v) in theta (ratio logits, log mean, log cv; index 3k + q): one device pass
    (pc_smooth_gauss_newton gives the system in (ratio, mean, sd)) and the chain rule on the
    3K x 3K matrices."""
    prm = prob.params(th)
    f, A_p, g_p = prob.smooth.gauss_newton(prm, prob.target)
    D = param_jacobian(th, prm)
    Dt = D.transpose(1, 2)
    return f, Dt @ A_p @ D, (Dt @ g_p[..., None])[..., 0]


def levenberg_marquardt(prob, theta0, iters=40, lam0=1e-2, max_step=1.0, time_limit=None, graph=True):
    """Levenberg-Marquardt from every candidate at once on the residuals r_v = log(1 + E_v) -
    log(1 + C_v) of the smoothed form. One Gauss-Newton pass per iteration (the Jacobian
    kernel, reduced on the device to J^T J, J^T r and the loss) at the trial point, which is
    kept in the search box every search shares; a candidate keeps its step if its loss falls
    (damping / 3) and otherwise stays where it was (damping x 4). (Left free, the search
    leaves the box towards sd/mean near 0.007: expected counts a near-deterministic type
    fits as well, but whose cells divide in lockstep, so that single histograms of the
    plain simulator scatter far more than the target's.) Steps solve (J^T J + lam diag(J^T J)) d = -J^T r per candidate (9 x 9 for
    three types). On a GPU one iteration (the pass and every small tensor operation around
    it) is captured once into a CUDA graph before the clock starts and replayed; without a
    GPU, or if capture fails, iterations run eagerly with the same arithmetic."""
    lo, hi = prob.box()
    n, K = theta0.shape[0], theta0.shape[1]
    P = 3 * K
    eye = torch.eye(P, dtype=torch.float64, device=theta0.device)
    # state, updated in place by step()
    th = theta0.clone()
    lam = torch.full((n,), lam0, dtype=torch.float64, device=th.device)
    f, A, g = gauss_newton_system(prob, th)

    def step():
        d = torch.diagonal(A, dim1=1, dim2=2)
        Ad = A + torch.diag_embed(lam[:, None] * d) + 1e-12 * d.amax(1)[:, None, None] * eye
        st = torch.linalg.solve_ex(Ad, -g[..., None])[0][..., 0]
        st = torch.nan_to_num(st, nan=0.0, posinf=0.0, neginf=0.0).clamp(-max_step, max_step)
        th_new = torch.minimum(torch.maximum(th + st.reshape(n, K, 3), lo), hi)
        f2, A2, g2 = gauss_newton_system(prob, th_new)
        ok = f2 < f  # NaN losses are never accepted
        th.copy_(torch.where(ok[:, None, None], th_new, th))
        A.copy_(torch.where(ok[:, None, None], A2, A))
        g.copy_(torch.where(ok[:, None], g2, g))
        f.copy_(torch.where(ok, f2, f))
        lam.copy_(torch.where(ok, lam / 3.0, lam * 4.0).clamp(1e-7, 1e7))

    run = step
    if graph and th.is_cuda:
        try:
            side = torch.cuda.Stream()
            side.wait_stream(torch.cuda.current_stream())
            with torch.cuda.stream(side):
                step()  # warm-up outside capture (library scratch, solver workspaces)
            torch.cuda.current_stream().wait_stream(side)
            cg = torch.cuda.CUDAGraph()
            with torch.cuda.graph(cg):
                step()
            run = cg.replay
        except Exception:
            run = step
        th.copy_(theta0)
        lam.fill_(lam0)
    if th.is_cuda:
        torch.cuda.synchronize()
    t0 = time.perf_counter()
    f0, A0, g0 = gauss_newton_system(prob, th)
    f.copy_(f0)
    A.copy_(A0)
    g.copy_(g0)
    i = int(torch.argmin(f))
    best = float(f[i])
    trace = [(time.perf_counter() - t0, best)]
    snaps = [(trace[0][0], th[i].clone())]
    for _ in range(iters):
        run()
        i = int(torch.argmin(f))
        if float(f[i]) < best:
            best = float(f[i])
            snaps.append((time.perf_counter() - t0, th[i].clone()))
        trace.append((time.perf_counter() - t0, best))
        if time_limit and trace[-1][0] > time_limit:
            break
    return trace, snaps


def levenberg_marquardt_plain(prob, theta0, iters=40, lam0=1e-2, max_step=1.0, time_limit=None):
    """Levenberg-Marquardt steps from the smoothed form's Gauss-Newton system, accepted where
    the plain simulator's own loss (all candidates as one batch, one seed for all: common
    random numbers) falls: a derivative-based search on the simulator's loss. Each iteration
    is one Gauss-Newton pass and one batch run; it sees what the smoothed loss cannot, the
    scatter of single stochastic histograms."""
    lo, hi = prob.box()
    n, K = theta0.shape[0], theta0.shape[1]
    P = 3 * K
    eye = torch.eye(P, dtype=torch.float64, device=theta0.device)
    th = theta0.clone()
    lam = torch.full((n,), lam0, dtype=torch.float64, device=th.device)
    if th.is_cuda:
        torch.cuda.synchronize()
    t0 = time.perf_counter()
    f = prob.loss_plain(th)
    _, A, g = gauss_newton_system(prob, th)
    i = int(torch.argmin(f))
    best = float(f[i])
    trace = [(time.perf_counter() - t0, best)]
    snaps = [(trace[0][0], th[i].clone())]
    for _ in range(iters):
        d = torch.diagonal(A, dim1=1, dim2=2)
        Ad = A + torch.diag_embed(lam[:, None] * d) + 1e-12 * d.amax(1)[:, None, None] * eye
        st = torch.linalg.solve_ex(Ad, -g[..., None])[0][..., 0]
        st = torch.nan_to_num(st, nan=0.0, posinf=0.0, neginf=0.0).clamp(-max_step, max_step)
        th_new = torch.minimum(torch.maximum(th + st.reshape(n, K, 3), lo), hi)
        f2 = prob.loss_plain(th_new)
        _, A2, g2 = gauss_newton_system(prob, th_new)
        ok = f2 < f
        th = torch.where(ok[:, None, None], th_new, th)
        A = torch.where(ok[:, None, None], A2, A)
        g = torch.where(ok[:, None], g2, g)
        f = torch.where(ok, f2, f)
        lam = torch.where(ok, lam / 3.0, lam * 4.0).clamp(1e-7, 1e7)
        i = int(torch.argmin(f))
        if float(f[i]) < best:
            best = float(f[i])
            snaps.append((time.perf_counter() - t0, th[i].clone()))
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
    g = torch.Generator(device=theta0.device).manual_seed(seed)
    lo, hi = prob.box()
    x = theta0.clone()
    vel = torch.zeros_like(x)
    vmax = 0.5 * (hi - lo)
    with torch.no_grad():
        if x.is_cuda:
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


def neutral_trace(prob, snaps, n_seeds):
    """(time, model-neutral loss of the search's best parameters so far) per snapshot."""
    if not snaps:
        return []
    L = prob.loss_plain_mean(torch.stack([th for _, th in snaps]), n_seeds)
    return [(t, float(v)) for (t, _), v in zip(snaps, L)]


def compare(engine, candidates=256, seed=7, gd_iters=300, pso_seconds=40.0, paths=2, lm_iters=40,
            full=True, neutral_seeds=16):
    """Derivative-based searches on the smoothed form (Levenberg-Marquardt with the forward-
    mode Jacobian; Adam with the adjoint gradient) against particle swarms (on the smoothed
    form, and on the plain simulator through the batched form), all from one population,
    all scored afterwards with the same accurate loss. The headline level is the worse of
    the plain-simulator swarm's and Levenberg-Marquardt's final accurate losses (a level
    both reach); the ratio is the swarm's time to reach it over Levenberg-Marquardt's.
    With neutral_seeds > 0 the snapshots of those two searches are also scored with the
    plain simulator's loss averaged over that many seeds, and the same ratio is formed on
    that scale. full=False runs only Levenberg-Marquardt and the plain-simulator swarm."""
    prob = Problem(engine, seed=seed, paths=paths)
    theta0 = prob.start(candidates, seed)
    levenberg_marquardt(prob, theta0, iters=3)  # warm-up of every code path
    if full:
        gradient_descent(prob, theta0, iters=3)
        particle_swarm(prob, theta0, iters=3)
    particle_swarm(prob, theta0, iters=2, loss=prob.loss_plain)
    levenberg_marquardt_plain(prob, theta0, iters=2)
    lm, lm_snaps = levenberg_marquardt(prob, theta0, iters=lm_iters)
    lmp, lmp_snaps = levenberg_marquardt_plain(prob, theta0, iters=3 * lm_iters)
    gd = gd_snaps = ps = ps_snaps = None
    if full:
        gd, gd_snaps = gradient_descent(prob, theta0, iters=gd_iters)
        ps, ps_snaps = particle_swarm(prob, theta0, iters=1_000_000, time_limit=pso_seconds)
    pp, pp_snaps = particle_swarm(prob, theta0, iters=1_000_000, time_limit=pso_seconds, loss=prob.loss_plain)
    acc_lm, acc_pp = accurate_trace(prob, lm_snaps), accurate_trace(prob, pp_snaps)
    acc_gd = accurate_trace(prob, gd_snaps) if full else []
    acc_ps = accurate_trace(prob, ps_snaps) if full else []
    with torch.no_grad():
        hidden = torch.tensor([prob.hidden], dtype=torch.float64, device="cuda")
        th_h = torch.stack([torch.log(hidden[0, :, 0]), torch.log(hidden[0, :, 1]),
                            torch.log(hidden[0, :, 2] / hidden[0, :, 1])], dim=-1)[None]
        l_true = float(prob.loss_accurate(th_h)[0])

    def best_final(tr):
        return min(l for _, l in tr) if tr else None

    head = max(best_final(acc_pp), best_final(acc_lm))
    # the equal loss, and fixed multiples of the hidden parameters' own loss
    levels = sorted({head} | {f * l_true for f in (1.5, 1.25, 1.1, 1.05, 1.025, 1.0)}, reverse=True)
    table = []
    for L in levels:
        tl, tg = first_below(acc_lm, L), first_below(acc_gd, L)
        tp, ts = first_below(acc_pp, L), first_below(acc_ps, L)
        table.append({"accurate_loss": L, "lm_seconds": tl, "gd_seconds": tg, "pso_plain_seconds": tp,
                      "pso_smooth_seconds": ts, "ratio_plain": (tp / tl) if (tl and tp) else None,
                      "ratio_smooth": (ts / tl) if (tl and ts) else None})
    tl, tp = first_below(acc_lm, head), first_below(acc_pp, head)
    neutral = None
    if neutral_seeds:
        n_lm, n_pp = neutral_trace(prob, lm_snaps, neutral_seeds), neutral_trace(prob, pp_snaps, neutral_seeds)
        n_lmp = neutral_trace(prob, lmp_snaps, neutral_seeds)
        n_true = float(prob.loss_plain_mean(th_h, neutral_seeds)[0])
        head_n = max(best_final(n_pp), best_final(n_lm))
        tln, tpn = first_below(n_lm, head_n), first_below(n_pp, head_n)
        head_p = max(best_final(n_pp), best_final(n_lmp))
        tlp, tpp = first_below(n_lmp, head_p), first_below(n_pp, head_p)
        nlevels = []
        for f in (1.5, 1.25, 1.1, 1.05):
            L = f * n_true
            a, b = first_below(n_lm, L), first_below(n_pp, L)
            nlevels.append({"plain_loss": L, "lm_seconds": a, "pso_plain_seconds": b,
                            "ratio_plain": (b / a) if (a and b) else None})
        neutral = {"seeds": neutral_seeds, "plain_loss_at_hidden": n_true,
                   "lm_best": best_final(n_lm), "pso_plain_best": best_final(n_pp),
                   "equal_loss": head_n, "gradient_seconds_to_equal_loss": tln,
                   "pso_seconds_to_equal_loss": tpn, "speedup": (tpn / tln) if (tln and tpn) else None,
                   "levels": nlevels,
                   "lm_plain": {"best": best_final(n_lmp), "iters": len(lmp) - 1, "seconds": lmp[-1][0],
                                "equal_loss": head_p, "seconds_to_equal_loss": tlp,
                                "pso_seconds_to_equal_loss": tpp,
                                "speedup": (tpp / tlp) if (tlp and tpp) else None,
                                "method": "Levenberg-Marquardt steps from the smoothed form's Gauss-Newton system, "
                                          "accepted on the plain simulator's loss (one batch per iteration)"},
                   "what": "mean plain-simulator loss over %d independent seeds of each snapshot" % neutral_seeds}
    return {
        "seed": seed,
        "candidates": candidates,
        "lineages_per_cell": paths,
        "hidden": prob.hidden,
        "accurate_loss_at_hidden": l_true,
        "lm": {"iters": len(lm) - 1, "seconds": lm[-1][0], "best_smoothed_loss": lm[-1][1],
               "best_accurate_loss": best_final(acc_lm),
               "seconds_per_iter": lm[-1][0] / max(1, len(lm) - 1),
               "method": "Levenberg-Marquardt on the smoothed form, one Gauss-Newton pass (Jacobian kernel "
                         "reduced on the device) per iteration"},
        "gd": None if gd is None else {
            "iters": len(gd), "seconds": gd[-1][0], "best_smoothed_loss": gd[-1][1],
            "best_accurate_loss": best_final(acc_gd), "method": "Adam on the smoothed form, cosine lr 0.1 -> 0.002"},
        "pso_smooth": None if ps is None else {
            "iters": len(ps) - 1, "seconds": ps[-1][0], "best_smoothed_loss": ps[-1][1],
            "best_accurate_loss": best_final(acc_ps),
            "method": "particle swarm on the smoothed form (constriction, ring neighbourhood)"},
        "pso_plain": {"iters": len(pp) - 1, "seconds": pp[-1][0], "best_plain_loss": pp[-1][1],
                      "best_accurate_loss": best_final(acc_pp),
                      "method": "particle swarm on the plain simulator, candidates as the instances of one batch "
                                "(set_types + run + totals per iteration)"},
        "equal_loss": head,
        "equal_loss_is": "accurate loss both Levenberg-Marquardt and the plain-simulator swarm reach",
        "gradient_seconds_to_equal_loss": tl,
        "pso_seconds_to_equal_loss": tp,
        "speedup": (tp / tl) if (tl and tp) else None,
        "levels": table,
        "model_neutral": neutral,
        "traces": {"lm": acc_lm, "gd": acc_gd, "pso_plain": acc_pp},
    }


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--candidates", type=int, default=256)
    ap.add_argument("--seed", type=int, default=7)
    ap.add_argument("--gd-iters", type=int, default=300)
    ap.add_argument("--pso-seconds", type=float, default=40.0)
    ap.add_argument("--paths", type=int, default=2)
    ap.add_argument("--lm-iters", type=int, default=40)
    a = ap.parse_args()
    from . import Engine
    eng = Engine(0)
    print(json.dumps(compare(eng, a.candidates, a.seed, a.gd_iters, a.pso_seconds, a.paths, a.lm_iters)))


if __name__ == "__main__":
    main()
