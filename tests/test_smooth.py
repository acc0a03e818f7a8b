"""The smoothed, differentiable form: forward, hand-written adjoint, torch.autograd.Function.

Checks: (1) the adjoint against central finite differences of the forward (relative step
1e-4, common random numbers: the same seed, so the same lineages and normals), within 1e-3
relative; (2) expected counts and their gradients against the analytic Gaussian-sum model
at sd/mean = 0.1: conditional on the initial age U, S_g ~ N(mean (g + U), sd^2 ((1 + U)^2 +
g - 1)), and E[sigmoid((T - S) / h)] = P(S + Logistic(0, h) <= T), integrated by quadrature.
The kernel's leaf weight s_1 ... s_g (1 - s_{g+1}) equals s_g - s_{g+1} up to terms of order
exp(-mean / h) (= e^-48 here), so E_g = 2^g (P_g - P_{g+1}) is the analytic reference;
(3) the autograd wrapper and determinism.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


def calib_bins(n_bins=256, cells=100_000, seed=5):
    rng = np.random.default_rng(seed)
    v = np.exp(rng.uniform(np.log(1.0), np.log(1e4), n_bins))
    f = rng.multinomial(cells, np.full(n_bins, 1.0 / n_bins))
    return [(float(a), int(b)) for a, b in zip(v, f)]


def loss_fn(E, target):
    return ((torch.log1p(E) - torch.log1p(target)) ** 2).sum(dim=1)


@pytest.fixture(scope="module")
def smooth_setup(engine):
    from procell.smooth import Smooth
    bins = calib_bins()
    sm = Smooth(engine, bins, n_types=3, t_max=168.0, phi=None, h=0.5, paths=2, seed=11)
    yield sm, bins
    sm.close()


def params_tensor(rows):
    return torch.tensor(rows, dtype=torch.float64, device="cuda")


BASE = [[[0.5, 40.0, 8.0], [0.3, 60.0, 15.0], [0.2, 90.0, 20.0]],
        [[0.2, 35.0, 3.5], [0.45, 55.0, 5.5], [0.35, 80.0, 8.0]]]


def test_adjoint_matches_central_differences(smooth_setup):
    sm, _ = smooth_setup
    P = params_tensor(BASE)
    # a target histogram that is not the model itself, so the loss gradient is nonzero
    target = sm.forward(params_tensor([[[0.4, 45.0, 9.0], [0.4, 58.0, 12.0], [0.2, 85.0, 17.0]]])).repeat(2, 1)
    E = sm.forward(P)
    L = loss_fn(E, target)
    gE = 2.0 * (torch.log1p(E) - torch.log1p(target)) / (1.0 + E)
    grad = sm.backward(P, gE).cpu().numpy()
    # central differences: every (candidate, type, parameter) perturbed by +-1e-4 relative,
    # all in one batch of candidates
    C, K = P.shape[0], P.shape[1]
    rows, steps = [], []
    for c in range(C):
        for k in range(K):
            for q in range(3):
                d = 1e-4 * abs(float(P[c, k, q]))
                for sgn in (1.0, -1.0):
                    Q = P[c].clone()
                    Q[k, q] += sgn * d
                    rows.append(Q)
                steps.append(d)
    Pf = torch.stack(rows)
    tf = target[:1].expand(Pf.shape[0], -1)
    Lf = loss_fn(sm.forward(Pf), tf).cpu().numpy()
    fd = ((Lf[0::2] - Lf[1::2]) / (2.0 * np.array(steps))).reshape(C, K, 3)
    sm.sync()
    assert np.all(np.isfinite(grad)) and np.all(np.isfinite(fd))
    scale = np.abs(fd).max()
    err = np.abs(grad - fd)
    assert np.all(err <= 1e-3 * np.abs(fd) + 1e-6 * scale), (grad, fd, err / np.abs(fd))


def _gauss_logistic_cdf(T, m, s, h, nodes=160):
    """E[sigmoid((T - m - s X) / h)], X ~ N(0, 1), by Gauss-Hermite quadrature, and its
    derivatives with respect to m and s."""
    x, w = np.polynomial.hermite_e.hermegauss(nodes)
    w = w / np.sqrt(2.0 * np.pi)
    a = (T - m[..., None] - s[..., None] * x) / h
    sig = 1.0 / (1.0 + np.exp(-a))
    dsig = sig * (1.0 - sig) / h
    return (sig * w).sum(-1), (-dsig * w).sum(-1), (-dsig * x * w).sum(-1)


def analytic_counts(mu, sd, T, h, gens):
    """Expected leaves per initial cell at generations 0..gens-1 (no phi cap in reach) and
    d/d mean, d/d sd, for the smoothed model with untruncated normal division times."""
    u, wu = np.polynomial.legendre.leggauss(64)
    u = 0.5 * (u + 1.0)
    wu = 0.5 * wu
    P = np.zeros(gens + 1)
    dPm = np.zeros(gens + 1)
    dPs = np.zeros(gens + 1)
    P[0] = 1.0
    for g in range(1, gens + 1):
        m = mu * (g + u)
        var_c = (1.0 + u) ** 2 + g - 1.0
        s = sd * np.sqrt(var_c)
        p, dm, ds = _gauss_logistic_cdf(T, m, s, h)
        P[g] = (p * wu).sum()
        dPm[g] = (dm * (g + u) * wu).sum()
        dPs[g] = (ds * np.sqrt(var_c) * wu).sum()
    pw = 2.0 ** np.arange(gens)
    E = pw * (P[:-1] - P[1:])
    dEm = pw * (dPm[:-1] - dPm[1:])
    dEs = pw * (dPs[:-1] - dPs[1:])
    return E, dEm, dEs


def test_gaussian_sum_model(engine):
    from procell.smooth import Smooth
    mu, sd, T, h = 24.0, 2.4, 100.0, 0.5
    value, cells, paths = 2.0 ** 30, 400_000, 4  # one bin; the phi cap (30) is never reached
    sm = Smooth(engine, [(value, cells)], n_types=1, t_max=T, phi=1.0, h=h, paths=paths, seed=3)
    gens = 7
    E_a, dEm_a, dEs_a = analytic_counts(mu, sd, T, h, gens)
    P = params_tensor([[[1.0, mu, sd]]])
    E = sm.forward(P)[0].cpu().numpy() / cells
    vals = sm.values
    idx = [int(np.searchsorted(vals, value / 2 ** g)) for g in range(gens)]
    E_mc = E[idx]
    main = E_a > 0.02 * E_a.max()
    assert np.all(np.abs(E_mc[main] - E_a[main]) <= 0.02 * E_a[main] + 0.005 * E_a.max()), (E_mc, E_a)
    # gradients of each generation's expected count: upstream gradient = one-hot on its value
    for g in np.flatnonzero(main):
        gE = torch.zeros(1, sm.n_values, dtype=torch.float64, device="cuda")
        gE[0, idx[g]] = 1.0 / cells
        grad = sm.backward(P, gE)[0, 0].cpu().numpy()
        assert abs(grad[1] - dEm_a[g]) <= 0.03 * abs(dEm_a).max(), (g, grad, dEm_a[g])
        assert abs(grad[2] - dEs_a[g]) <= 0.03 * abs(dEs_a).max() + 1e-4, (g, grad, dEs_a[g])
        assert abs(grad[0] - E_a[g]) <= 0.02 * E_a[g]  # d/d ratio = the count itself
    sm.sync()
    sm.close()


def test_lineage_draws_kept_or_redrawn_give_identical_results(engine, smooth_setup):
    """A smoothed plan draws its lineages' normals and initial ages once and keeps them in HBM
    (option smooth_predraw, the default); with the option off every pass draws them again.
    Forward, adjoint and Jacobian must not change by a single bit."""
    from procell.smooth import Smooth
    sm, bins = smooth_setup
    engine.set_option("smooth_predraw", 0)
    try:
        redraw = Smooth(engine, bins, n_types=3, t_max=168.0, phi=None, h=0.5, paths=2, seed=11)
    finally:
        engine.set_option("smooth_predraw", 1)
    try:
        P = params_tensor(BASE)
        gE = torch.tensor(np.random.default_rng(3).normal(size=(2, sm.n_values)), device="cuda")
        for a, b in ((sm.forward(P), redraw.forward(P)), (sm.backward(P, gE), redraw.backward(P, gE))):
            assert torch.equal(a, b)
        (Ea, Ja), (Eb, Jb) = sm.jacobian(P), redraw.jacobian(P)
        assert torch.equal(Ea, Eb) and torch.equal(Ja, Jb)
        sm.sync()
    finally:
        redraw.close()


def test_autograd_function_and_determinism(smooth_setup):
    from procell.smooth import expected_counts
    sm, _ = smooth_setup
    P = params_tensor(BASE).requires_grad_(True)
    target = torch.full((2, sm.n_values), 3.0, dtype=torch.float64, device="cuda")
    E = expected_counts(sm, P)
    loss = loss_fn(E, target).sum()
    loss.backward()
    gE = 2.0 * (torch.log1p(E.detach()) - torch.log1p(target)) / (1.0 + E.detach())
    direct = sm.backward(P.detach(), gE)
    assert torch.equal(P.grad, direct)
    E2 = sm.forward(P.detach())
    assert torch.equal(E.detach(), E2)
    sm.sync()


def test_many_types_match_cpu_restatement(engine):
    """Six types (one quiescent, one zero-mean) and 37 candidates (two partial groups of 32):
    forward, adjoint and Jacobian of the per-type grids against the CPU restatement."""
    import smooth_ref
    from procell.smooth import Smooth
    bins = [(300.0, 14), (45.0, 9), (7.5, 11), (2.2, 6)]
    t_max, phi, h, paths, seed = 120.0, 1.0, 0.7, 2, 4242
    rng = np.random.default_rng(8)
    C, K = 37, 6
    params = []
    for c in range(C):
        r = rng.dirichlet(np.ones(K))
        rows = [[float(r[k]), float(rng.uniform(18, 70)), float(rng.uniform(1, 12))] for k in range(K)]
        rows[1][1:] = [-1.0, -1.0]   # quiescent
        rows[4][1:] = [0.0, 3.0]     # zero mean: never due
        params.append(rows)
    sm = Smooth(engine, bins, n_types=K, t_max=t_max, phi=phi, h=h, paths=paths, seed=seed)
    gE = rng.normal(size=(C, sm.n_values))
    E_ref, G_ref, vals, J_ref = smooth_ref.forward_backward(bins, t_max, phi, h, paths, seed, params, gE,
                                                            with_jacobian=True)
    P = params_tensor(params)
    E = sm.forward(P).cpu().numpy()
    G = sm.backward(P, torch.tensor(gE, device="cuda")).cpu().numpy()
    EJ, J = (x.cpu().numpy() for x in sm.jacobian(P))
    sm.sync()
    sm.close()
    assert np.array_equal(vals, sm.values)
    assert np.allclose(E, E_ref, rtol=2e-5, atol=1e-9 * np.abs(E_ref).max())
    assert np.allclose(EJ, E_ref, rtol=2e-5, atol=1e-9 * np.abs(E_ref).max())
    assert np.allclose(G, G_ref, rtol=2e-5, atol=1e-7 * np.abs(G_ref).max())
    assert np.allclose(J, J_ref, rtol=2e-5, atol=1e-7 * np.abs(J_ref).max())


@pytest.mark.parametrize("K", [3, 8])
def test_gauss_newton_matches_jacobian(engine, K):
    """pc_smooth_gauss_newton (loss, J^T J, J^T r of the squared log-count loss, reduced on
    the device) against the same quantities formed from pc_smooth_jacobian; K = 8 uses every
    output slot of the reduction (24 parameters: 300 + 24 + 1 outputs per candidate)."""
    from procell.smooth import Smooth
    bins = calib_bins(n_bins=40, cells=4000, seed=9)
    sm = Smooth(engine, bins, n_types=K, t_max=150.0, phi=None, h=0.5, paths=2, seed=21)
    rng = np.random.default_rng(K)
    C = 45
    params = []
    for c in range(C):
        r = rng.dirichlet(np.ones(K))
        params.append([[float(r[k]), float(rng.uniform(25, 90)), float(rng.uniform(2, 15))] for k in range(K)])
    if K > 2:
        params[3][1][1:] = [-1.0, -1.0]
    P = params_tensor(params)
    target = sm.forward(P[:1])[0] * 1.3 + 2.0
    f, A, g = sm.gauss_newton(P, target)
    E, J = sm.jacobian(P)
    sm.sync()
    sm.close()
    Jv = J.reshape(C, sm.n_values, 3 * K) / (1.0 + E)[..., None]
    r = torch.log1p(E) - torch.log1p(target)
    assert torch.allclose(f, (r * r).sum(1), rtol=1e-12, atol=0)
    A_ref = Jv.transpose(1, 2) @ Jv
    g_ref = (Jv * r[..., None]).sum(1)
    assert torch.allclose(A, A_ref, rtol=1e-10, atol=1e-13 * float(A_ref.abs().max()))
    assert torch.allclose(g, g_ref, rtol=1e-10, atol=1e-13 * float(g_ref.abs().max()))
    assert torch.equal(A, A.transpose(1, 2))


def test_candidate_order_does_not_change_results(smooth_setup):
    """Kernels visit each type's candidates in order of that type's mean; a candidate's
    results are the same bits wherever it sits in the batch."""
    sm, _ = smooth_setup
    g = torch.Generator(device="cuda").manual_seed(3)
    n = 70  # not a multiple of 32
    P = torch.stack([torch.rand(n, 3, generator=g, device="cuda", dtype=torch.float64) * 0.9 + 0.05,
                     torch.rand(n, 3, generator=g, device="cuda", dtype=torch.float64) * 80.0 + 25.0,
                     torch.rand(n, 3, generator=g, device="cuda", dtype=torch.float64) * 10.0 + 1.0], dim=-1)
    P[5, 1, 1] = -1.0   # a quiescent type
    P[9] = P[4]         # equal means (ties)
    perm = torch.randperm(n, generator=g, device="cuda")
    E, Ep = sm.forward(P), sm.forward(P[perm])
    gE = torch.rand(n, sm.n_values, generator=g, device="cuda", dtype=torch.float64)
    G, Gp = sm.backward(P, gE), sm.backward(P[perm], gE[perm])
    (EJ, J), (EJp, Jp) = sm.jacobian(P), sm.jacobian(P[perm])
    sm.sync()
    assert torch.equal(E[perm], Ep) and torch.equal(G[perm], Gp)
    assert torch.equal(EJ[perm], EJp) and torch.equal(J[perm], Jp)
    assert torch.equal(E[9], E[4])


def test_quiescent_type_counts_at_generation_zero(engine):
    from procell.smooth import Smooth
    sm = Smooth(engine, [(100.0, 1000), (0.5, 200)], n_types=2, t_max=50.0, phi=1.0, h=0.5, paths=1, seed=1)
    P = params_tensor([[[0.25, -1.0, -1.0], [0.75, 1e6, 1.0]]])  # the second type never divides by t_max
    E = sm.forward(P)[0].cpu().numpy()
    # value 100 (countable): every cell is a generation-0 leaf; value 0.5 < phi: not counted
    i100 = int(np.searchsorted(sm.values, 100.0))
    assert abs(E[i100] - 1000.0) < 1e-6 and abs(E.sum() - 1000.0) < 1e-6
    sm.sync()
    sm.close()


def test_matches_cpu_restatement(engine):
    """Expected counts and gradients against oracle/smooth_ref.py (FP64, independent)."""
    import smooth_ref
    from procell.smooth import Smooth
    bins = [(640.0, 60), (37.0, 45), (3.0, 20), (1500.0, 0), (9.5, 30), (0.7, 10)]
    t_max, phi, h, paths, seed = 150.0, 1.0, 0.5, 2, 123456789012
    params = [[[0.5, 30.0, 6.0], [0.3, 45.0, 18.0], [0.2, -1.0, -1.0]],
              [[0.6, 25.0, 12.0], [0.4, 0.0, 1.0], [0.0, 40.0, 4.0]]]
    rng = np.random.default_rng(0)
    sm = Smooth(engine, bins, n_types=3, t_max=t_max, phi=phi, h=h, paths=paths, seed=seed)
    gE = rng.normal(size=(2, sm.n_values))
    E_ref, G_ref, vals = smooth_ref.forward_backward(bins, t_max, phi, h, paths, seed, params, gE)
    assert np.array_equal(vals, sm.values)
    P = params_tensor(params)
    E = sm.forward(P).cpu().numpy()
    G = sm.backward(P, torch.tensor(gE, device="cuda")).cpu().numpy()
    sm.sync()
    sm.close()
    assert np.allclose(E, E_ref, rtol=2e-5, atol=1e-9 * np.abs(E_ref).max()), np.abs(E - E_ref).max()
    assert np.allclose(G, G_ref, rtol=2e-5, atol=1e-7 * np.abs(G_ref).max()), (G, G_ref)


def test_jacobian_matches_cpu_restatement_and_adjoint(engine):
    """The forward-mode Jacobian kernel: its expected counts equal the forward kernel's, its
    contraction with any upstream gradient equals the adjoint, and it matches the FP64 CPU
    restatement entry by entry."""
    import smooth_ref
    from procell.smooth import Smooth
    bins = [(640.0, 60), (37.0, 45), (3.0, 20), (1500.0, 0), (9.5, 30), (0.7, 10)]
    t_max, phi, h, paths, seed = 150.0, 1.0, 0.5, 2, 987654321
    params = [[[0.5, 30.0, 6.0], [0.3, 45.0, 18.0], [0.2, -1.0, -1.0]],
              [[0.6, 25.0, 12.0], [0.4, 0.0, 1.0], [0.0, 40.0, 4.0]]]
    sm = Smooth(engine, bins, n_types=3, t_max=t_max, phi=phi, h=h, paths=paths, seed=seed)
    gE = np.random.default_rng(1).normal(size=(2, sm.n_values))
    E_ref, G_ref, vals, J_ref = smooth_ref.forward_backward(bins, t_max, phi, h, paths, seed, params, gE,
                                                            with_jacobian=True)
    assert np.array_equal(vals, sm.values)
    P = params_tensor(params)
    E, J = sm.jacobian(P)
    E_fwd = sm.forward(P)
    G = sm.backward(P, torch.tensor(gE, device="cuda"))
    sm.sync()
    sm.close()
    E, J, E_fwd, G = (x.cpu().numpy() for x in (E, J, E_fwd, G))
    assert np.allclose(J, J_ref, rtol=2e-5, atol=1e-7 * np.abs(J_ref).max()), np.abs(J - J_ref).max()
    assert np.allclose(E, E_ref, rtol=2e-5, atol=1e-9 * np.abs(E_ref).max())
    assert np.allclose(E, E_fwd, rtol=1e-5, atol=1e-9 * np.abs(E).max())
    GJ = np.einsum("cv,cvkq->ckq", gE, J)
    assert np.allclose(GJ, G, rtol=1e-4, atol=1e-6 * np.abs(G).max()), (GJ, G)
    # the ratio column of a zero-ratio type is still its (unscaled) contribution
    assert J[1, :, 2, 0].sum() > 0 and np.all(J[1, :, 2, 1:] == 0)


def test_jacobian_matches_central_differences(smooth_setup):
    sm, _ = smooth_setup
    P = params_tensor(BASE)
    E, J = sm.jacobian(P)
    C, K = P.shape[0], P.shape[1]
    rows, steps = [], []
    for c in range(C):
        for k in range(K):
            for q in range(3):
                d = 1e-4 * abs(float(P[c, k, q]))
                for sgn in (1.0, -1.0):
                    Q = P[c].clone()
                    Q[k, q] += sgn * d
                    rows.append(Q)
                steps.append(d)
    Ef = sm.forward(torch.stack(rows)).cpu().numpy()
    sm.sync()
    fd = ((Ef[0::2] - Ef[1::2]) / (2.0 * np.array(steps))[:, None]).reshape(C, K, 3, -1).transpose(0, 3, 1, 2)
    J = J.cpu().numpy()
    assert np.all(np.isfinite(J))
    # every Jacobian column (candidate, type, parameter) against its central difference, in
    # norm over the values (single entries of the difference carry the forward's FP32
    # rounding divided by the step)
    err = np.linalg.norm(J - fd, axis=1) / np.linalg.norm(fd, axis=1)
    assert np.all(err <= 1e-3), err


def test_converges_to_plain_expectation(engine):
    """With many lineages per cell (independent replicas) and a small h, the expected counts
    approach the plain form's histogram averaged over seeds."""
    from procell.smooth import Smooth
    bins = [(100.0, 300), (37.5, 200), (700.0, 100)]
    types = [(0.6, 40.0, 8.0), (0.4, 55.0, 5.5)]
    T, phi = 168.0, 1.0
    runs = 64
    avg = sum(engine.simulate(bins, types, T, phi, 9000 + s).totals.astype(np.float64) for s in range(runs)) / runs
    sm = Smooth(engine, bins, n_types=2, t_max=T, phi=phi, h=0.05, paths=256, seed=4)
    E = sm.forward(params_tensor([types]))[0].cpu().numpy()
    sm.sync()
    sm.close()
    assert abs(E.sum() - avg.sum()) <= 0.01 * avg.sum()
    big = avg > 0.05 * avg.max()
    # Monte Carlo error of both sides is a few percent at these counts
    assert np.all(np.abs(E[big] - avg[big]) <= 0.06 * avg[big] + 5.0), np.c_[E[big], avg[big]]
