"""CPU checks of the oracle (the CPU restatement the GPU engine is compared against).

Pins: the published Philox4x32-10 known-answer vectors (Random123 distribution), the
ziggurat construction's invariants and the statistics of the normal it produces, and
hand-derivable outcomes of the reference's rules (src/simulation/proliferation.cu:315-410,
src/simulation/cell.cu:25-143, src/io/parser.cu:68-154).
"""
import math

import numpy as np
import pytest
from scipy import stats


def test_philox_known_answers(oracle_lib):
    # Random123 kat_vectors, philox4x32 with 10 rounds: (counter, key) -> output
    kat = [
        ([0, 0, 0, 0], [0, 0], [0x6627E8D5, 0xE169C58D, 0xBC57AC4C, 0x9B00DBD8]),
        ([0xFFFFFFFF] * 4, [0xFFFFFFFF] * 2, [0x408F276D, 0x41C83B0E, 0xA20BC7C6, 0x6D5451FD]),
        ([0x243F6A88, 0x85A308D3, 0x13198A2E, 0x03707344], [0xA4093822, 0x299F31D0],
         [0xD16CFE09, 0x94FDCCEB, 0x5001E420, 0x24126EA1]),
    ]
    for ctr, key, want in kat:
        assert oracle_lib.philox(ctr, key) == want


def test_ziggurat_tables(oracle_lib):
    k, w, f = oracle_lib.tables()
    n = len(k)
    assert n == 1024 and len(f) == n + 1
    r, v = 4.0388498461095045227, 1.2263246463530880729e-3
    x = w.astype(np.float64) * 2.0 ** 31
    # layer 1's right edge is r, edges shrink towards the top layer
    assert abs(x[1] - r) < 1e-6
    assert np.all(np.diff(x[1:]) < 0)
    assert k[n - 1] == 0 and f[n] == 1.0
    # every layer i >= 1 has area v: x_i * (f(x_{i+1}) - f(x_i))
    fx = np.exp(-0.5 * x[1:] ** 2)
    fnext = np.append(fx[1:], 1.0)
    areas = x[1:] * (fnext - fx)
    # x_i is rebuilt from the FP32-rounded w, and the difference f(x_{i+1}) - f(x_i) of a thin
    # layer amplifies that rounding: up to 8.5e-5 relative with 1024 layers (the tables are
    # built in FP64, where the construction closes to 4e-9)
    assert np.allclose(areas[:-1], v, rtol=2e-4), areas
    assert abs(areas[-1] - v) < 1e-3 * v
    # the base strip: rectangle [0, r] x [0, f(r)] plus the tail, area v
    tail = math.sqrt(math.pi / 2) * math.erfc(r / math.sqrt(2))
    assert abs(r * math.exp(-r * r / 2) + tail - v) < 1e-12
    # f tables agree with the density, fast-accept fractions with the edge ratios
    assert np.allclose(f[1:n], fx, rtol=1e-6)
    ratio = np.append(x[2:n] / x[1:n - 1], 0.0)
    assert np.allclose(k[1:n] / 2.0 ** 31, ratio, atol=1e-9)
    # about 99.57% of first attempts are accepted by the strip test alone (98.5% with 256
    # layers, 97.2% with 128); the proposals rejected overall are the area above the curve,
    # N v - sqrt(pi/2)
    assert 0.9955 < k.astype(np.float64).mean() / 2.0 ** 31 < 0.9960
    assert abs((n * v - math.sqrt(math.pi / 2)) / (n * v) - 0.001945) < 1e-5


def test_normal_statistics(oracle_lib):
    z = oracle_lib.normals(seed=2024, root=3, first_parent=0, count=1_000_000).astype(np.float64)
    assert abs(z.mean()) < 5 * 1 / math.sqrt(z.size)
    assert abs(z.var() - 1.0) < 5 * math.sqrt(2 / z.size)
    assert stats.kstest(z, "norm").pvalue > 1e-3
    # tails: P(|z| > 3) and P(|z| > 4) within 5 sigma of the binomial expectation
    for t in (3.0, 4.0):
        p = 2 * stats.norm.sf(t)
        n = np.sum(np.abs(z) > t)
        assert abs(n - p * z.size) < 5 * math.sqrt(p * z.size) + 2


def test_expf_logf_accuracy(oracle_lib):
    for x in np.linspace(-40, 0, 2001):
        got = oracle_lib.expf(float(np.float32(x)))
        want = math.exp(float(np.float32(x)))
        assert abs(got - want) <= 4e-7 * want + 1e-30
    for u in np.concatenate([np.geomspace(2 ** -24, 1.0, 2001), np.linspace(1e-3, 1, 999)]):
        uf = float(np.float32(u))
        assert abs(oracle_lib.logf(uf) - math.log(uf)) <= 3e-7 * max(1.0, abs(math.log(uf)))


def test_truncated_timer_positive(oracle_lib):
    # mean 1, sd 3: two thirds of first attempts are rejected; tau must stay > 0
    taus = [oracle_lib.tau(9, 5, p, c, 1.0, 3.0) for p in range(2000) for c in (0, 1)]
    assert min(taus) > 0
    # truncated normal mean: mu + sd * phi(a) / (1 - Phi(a)), a = -mu/sd
    a = -1.0 / 3.0
    want = 1.0 + 3.0 * stats.norm.pdf(a) / stats.norm.sf(a)
    assert abs(np.mean(taus) - want) < 5 * np.std(taus) / math.sqrt(len(taus))


def test_quiescent_only_reproduces_input(oracle_lib):
    bins = [(8.0, 3), (1.0, 5), (0.5, 2), (300.0, 0)]
    r = oracle_lib.simulate(bins, [(1.0, -1.0, -1.0)], t_max=100.0, phi=1.0, seed=1)
    got = {v: int(t) for v, t in zip(r.values, r.totals) if t}
    assert got == {1.0: 5, 8.0: 3}          # 0.5 < phi is never counted (proliferation.cu:353-381)
    assert r.stats["divisions"] == 0 and r.stats["uncounted"] == 2
    # value set: every nonzero bin halved while >= phi (parser.cu:126-137)
    assert list(r.values) == [1.0, 2.0, 4.0, 8.0]


def test_t_max_zero_means_no_division(oracle_lib):
    bins = [(64.0, 50), (3.0, 20)]
    r = oracle_lib.simulate(bins, [(0.5, 10.0, 2.0), (0.5, 20.0, 1.0)], t_max=0.0, phi=1.0, seed=3)
    assert r.stats["divisions"] == 0
    got = {v: int(t) for v, t in zip(r.values, r.totals) if t}
    assert got == {64.0: 50, 3.0: 20}


def test_deterministic_timer_single_division(oracle_lib):
    # sd = 0: tau = mu exactly. Root due time mu*(1+U), U in (0,1]; with t_max = 1.5 mu a root
    # divides iff U <= 1/2 and its daughters (due >= 2 mu) are leaves of generation 1.
    mu, n = 10.0, 4000
    r = oracle_lib.simulate([(64.0, n)], [(1.0, mu, 0.0)], t_max=1.5 * mu, phi=1.0, seed=11)
    c = {v: int(t) for v, t in zip(r.values, r.totals) if t}
    divided = c.get(32.0, 0) // 2
    assert c.get(32.0, 0) % 2 == 0
    assert c.get(64.0, 0) + divided == n
    assert abs(divided - n / 2) < 5 * math.sqrt(n / 4)
    assert r.stats["divisions"] == divided and r.stats["max_gen"] <= 1


def test_phi_boundary_blocks_division(oracle_lib):
    # f/2 > phi is strict: value 2*phi is due but cannot divide, so it vanishes
    # (proliferation.cu:323: no else branch, the cell is neither counted nor divided).
    r = oracle_lib.simulate([(2.0, 100)], [(1.0, 1.0, 0.1)], t_max=1e6, phi=1.0, seed=5)
    assert int(r.totals.sum()) == 0 and r.stats["vanished"] == 100
    # value 2*phi + tiny: divides once, daughters (phi + tiny/2) vanish
    v = 2.0 + 2 ** -40
    r = oracle_lib.simulate([(v, 10)], [(1.0, 1.0, 0.1)], t_max=1e6, phi=1.0, seed=5)
    assert r.stats["divisions"] == 10 and r.stats["vanished"] == 20


def test_complete_tree_counts(oracle_lib):
    # Every tree node either divides, is a leaf (counted or, for a root below phi,
    # uncounted) or vanishes, so roots + divisions == leaves + uncounted + vanished.
    bins = [(1024.0, 37), (3.0, 11), (0.25, 4)]
    types = [(0.6, 5.0, 1.5), (0.3, 9.0, 2.0), (0.1, -1.0, -1.0)]
    r = oracle_lib.simulate(bins, types, t_max=40.0, phi=0.5, seed=77)
    s = r.stats
    assert s["roots"] + s["divisions"] == s["leaves"] + s["uncounted"] + s["vanished"]
    assert int(r.totals.sum()) == s["leaves"]
    assert np.array_equal(r.per_type.sum(axis=1), r.totals)


def test_auto_phi_matches_reference_rule(oracle_lib):
    bins = [(5.0, 0), (3.0, 2), (7.0, 1)]
    a = oracle_lib.simulate(bins, [(1.0, 2.0, 0.5)], t_max=3.0, phi=None, seed=2)
    b = oracle_lib.simulate(bins, [(1.0, 2.0, 0.5)], t_max=3.0, phi=3.0, seed=2)
    assert np.array_equal(a.values, b.values) and np.array_equal(a.totals, b.totals)


def test_ratio_sum_check(oracle_lib):
    with pytest.raises(oracle_lib.OracleError, match="does not sum to 1"):
        oracle_lib.simulate([(4.0, 1)], [(0.5, 1.0, 0.1), (0.4, 2.0, 0.1)], t_max=1.0, phi=1.0)


def test_type_order_and_tracking(oracle_lib):
    # per-type columns are in file order; ratios drive the split of roots between types
    types = [(0.2, -1.0, -1.0), (0.8, -1.0, -1.0)]
    r = oracle_lib.simulate([(10.0, 20000)], types, t_max=1.0, phi=1.0, seed=8)
    row = r.per_type[list(r.values).index(10.0)]
    assert row.sum() == 20000
    assert abs(row[0] / 20000 - 0.2) < 0.02 and abs(row[1] / 20000 - 0.8) < 0.02


def test_threads_and_shards_are_deterministic(oracle_lib):
    import procell.configs as cfg
    w = cfg.small()
    a = oracle_lib.simulate(w.bins, w.types, w.t_max, w.phi, seed=w.seed, nthreads=1)
    b = oracle_lib.simulate(w.bins, w.types, w.t_max, w.phi, seed=w.seed, nthreads=7)
    assert np.array_equal(a.totals, b.totals) and a.stats == b.stats
    n = w.roots
    parts = [oracle_lib.simulate(w.bins, w.types, w.t_max, w.phi, seed=w.seed,
                                 root_begin=lo, root_end=hi)
             for lo, hi in ((0, n // 3), (n // 3, n - 5), (n - 5, n))]
    assert np.array_equal(sum(p.per_type for p in parts), a.per_type)


def test_smooth_restatement_adjoint_matches_central_differences(oracle_lib):
    """The CPU restatement of the smoothed form is itself differentiated correctly: its
    forward-mode gradient agrees with central differences of its own forward."""
    import smooth_ref
    bins = [(640.0, 12), (37.0, 9), (3.0, 5)]
    params = np.array([[[0.6, 30.0, 6.0], [0.4, 45.0, 18.0]]])
    nv = len(smooth_ref.prepare(bins, 1.0)[1])
    gE = np.random.default_rng(1).normal(size=(1, nv))
    E, G, vals = smooth_ref.forward_backward(bins, 150.0, 1.0, 0.5, 3, 99, params, gE)
    for k in range(2):
        for q in range(3):
            d = 1e-6 * abs(params[0, k, q])
            P1, P2 = params.copy(), params.copy()
            P1[0, k, q] += d
            P2[0, k, q] -= d
            E1, _, _ = smooth_ref.forward_backward(bins, 150.0, 1.0, 0.5, 3, 99, P1)
            E2, _, _ = smooth_ref.forward_backward(bins, 150.0, 1.0, 0.5, 3, 99, P2)
            fd = float((gE * (E1 - E2)).sum() / (2 * d))
            assert abs(G[0, k, q] - fd) <= 1e-5 * max(1.0, abs(fd)), (k, q, G[0, k, q], fd)


def test_smooth_restatement_jacobian(oracle_lib):
    """The restatement's Jacobian contracts to its adjoint and matches central differences
    of its own forward, column by column."""
    import smooth_ref
    bins = [(640.0, 12), (37.0, 9), (3.0, 5)]
    params = np.array([[[0.6, 30.0, 6.0], [0.4, 45.0, 18.0]]])
    nv = len(smooth_ref.prepare(bins, 1.0)[1])
    gE = np.random.default_rng(2).normal(size=(1, nv))
    E, G, _, J = smooth_ref.forward_backward(bins, 150.0, 1.0, 0.5, 3, 99, params, gE, with_jacobian=True)
    assert np.allclose(np.einsum("cv,cvkq->ckq", gE, J), G, rtol=1e-12, atol=1e-12 * np.abs(G).max())
    for k in range(2):
        for q in range(3):
            d = 1e-6 * abs(params[0, k, q])
            P1, P2 = params.copy(), params.copy()
            P1[0, k, q] += d
            P2[0, k, q] -= d
            E1, _, _ = smooth_ref.forward_backward(bins, 150.0, 1.0, 0.5, 3, 99, P1)
            E2, _, _ = smooth_ref.forward_backward(bins, 150.0, 1.0, 0.5, 3, 99, P2)
            fd = (E1 - E2)[0] / (2 * d)
            assert np.linalg.norm(J[0, :, k, q] - fd) <= 1e-5 * max(1.0, np.linalg.norm(fd)), (k, q)


def test_smooth_restatement_in_cpp_matches_python(oracle_lib):
    """The C++ restatement of the smoothed form (the benchmark's CPU baseline) equals the
    Python one: bit for bit on one thread, to summation order on several."""
    import smooth_ref
    bins = [(640.0, 30), (37.0, 25), (3.0, 12), (1500.0, 0), (9.5, 17), (0.7, 6)]
    params = [[[0.5, 30.0, 6.0], [0.3, 45.0, 18.0], [0.2, -1.0, -1.0]],
              [[0.6, 25.0, 12.0], [0.4, 0.0, 1.0], [0.0, 40.0, 4.0]]]
    nv = len(smooth_ref.prepare(bins, 1.0)[1])
    gE = np.random.default_rng(3).normal(size=(2, nv))
    E0, G0, _ = smooth_ref.forward_backward(bins, 150.0, 1.0, 0.5, 2, 987654321, params, gE)
    E1, G1 = oracle_lib.smooth(bins, 150.0, 1.0, 0.5, 2, 987654321, params, gE, nthreads=1)
    assert np.array_equal(E0, E1) and np.array_equal(G0, G1)
    E2, G2 = oracle_lib.smooth(bins, 150.0, 1.0, 0.5, 2, 987654321, params, gE, nthreads=4)
    assert np.allclose(E2, E0, rtol=1e-13, atol=1e-13 * np.abs(E0).max())
    assert np.allclose(G2, G0, rtol=1e-12, atol=1e-12 * np.abs(G0).max())
    E3, G3 = oracle_lib.smooth(bins, 150.0, None, 0.5, 1, 5, params[:1], nthreads=1)
    E4, _, _ = smooth_ref.forward_backward(bins, 150.0, None, 0.5, 1, 5, params[:1])
    assert G3 is None and np.array_equal(E3, E4)


def test_smooth_restatement_replica_zero_is_the_plain_tree(oracle_lib):
    """With one lineage per cell and h -> 0, a cell's smoothed weight is an unbiased estimate
    of its own plain-form tree: enumerating every path reproduces the oracle's counts."""
    import smooth_ref
    T, mu, sd, seed, cap = 168.0, 40.0, 8.0, 1234, 6
    res = oracle_lib.simulate([(100.0, 20)], [(1.0, mu, sd)], T, 1.0, seed=seed, nthreads=1)
    total = np.zeros(cap + 1)
    for r in range(20):
        R = oracle_lib.philox([0, 0, r, smooth_ref.PURPOSE_ROOT], [seed & 0xFFFFFFFF, seed >> 32])
        U = smooth_ref._unit53_open_closed(R[2], R[3])
        for bits in range(2 ** (cap + 1)):
            node, S = 1, 0.0
            for j in range(1, cap + 2):
                z = float(oracle_lib.normals(seed, r, node >> 1, 2)[node & 1])
                tau = sd * z + mu
                S = tau * U + tau if j == 1 else S + tau
                if S > T:
                    total[j - 1] += 2.0 ** (j - 1) / 2 ** (cap + 1)
                    break
                node = 2 * node + ((bits >> (j - 1)) & 1)
    assert np.allclose(total, res.per_type[::-1, 0], atol=1e-9)
