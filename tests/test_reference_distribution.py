"""The oracle against the reference binary, in distribution.

tests/golden/reference_*.json hold 64 runs each of the reference's own CUDA binary on the
small workload (written on a GPU machine by tests/golden/make_reference_fixtures.py). The
reference cannot be reproduced bit for bit (it draws from per-draw re-seeded curand states
with time-based seeds), so the comparison is statistical, with the run as the independent
unit: the leaves of one tree are correlated, so per-cell tests would be invalid. For each
output value, the mean count per run is compared (a chi-square-like sum of squared
standardised differences) and the pooled distribution of log-values is compared with a KS
statistic; both p-values come from 2000 permutations of the run labels.

* single type: the reference's generator defects cannot act on the type draw, and the
  oracle (hence the engine, which reproduces it bit for bit) agrees: p > 0.01 for both.
* two types: the reference draws a root's type and its first normal from the same freshly
  seeded generator state (src/simulation/cell.cu:81-122, both calls seeded with the same
  value), which couples type and first division time; its histogram differs from the
  documented model. The check records that signature: fewer roots out of time at
  generation 0 than independent draws give.
* two types sharing one timer (built for sm_100): the type drawn can no longer change any
  division time, so the totals must agree with the oracle, and they do; only the per-type
  columns (-r) still show the coupling: every root that stays undivided past t_max
  (generation 0) has type 0, none type 1. A type-1 root drew a uniform >= 0.53 for its type
  and its first normal from the same generator state, which bounds how long its first
  division can take. This isolates the two-type disagreement as that defect of the
  reference's generator, not a difference of the model.
* the medium histogram (1e6 initial cells) at t_max 150 with three types sharing one
  timer, the largest input the reference runs in one iteration with shared timers
  (tests/test_reference_planner.py): 16 runs of 2.5e6 leaves each. Totals agree within 3
  standard errors (a child grid the reference failed to launch would remove whole subtrees),
  and so do the per-value means; the pooled value distributions differ by at most 0.04% of
  the cells (a bound of 0.1% is asserted): at this sample size a KS test resolves even that,
  which the remaining per-draw reseeding of the reference (its initial-age uniform is drawn
  from seed * sd^2, src/simulation/cell.cu:124-143) accounts for.
"""
import json
import os

import numpy as np
import pytest

import procell.configs as cfg

HERE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def load(name):
    d = json.load(open(os.path.join(HERE, name)))
    keys = ["%.10g" % float.fromhex(v) for v in d["values"]]
    runs = [{k: c for k, c in zip(keys, row) if c} for row in d["counts"]]
    return d, runs


def oracle_runs(oracle_lib, w, n, base):
    out = []
    for k in range(n):
        o = oracle_lib.simulate(w.bins, w.types, w.t_max, w.phi, seed=base + k)
        out.append({"%.10g" % v: int(t) for v, t in zip(o.values, o.totals) if t})
    return out


def matrices(R, O):
    keys = sorted(set().union(*R, *O), key=float)
    A = np.array([[r.get(k, 0) for k in keys] for r in R], float)
    B = np.array([[r.get(k, 0) for k in keys] for r in O], float)
    logv = np.log(np.array([float(k) for k in keys]))
    keep = (A.sum(0) + B.sum(0)) >= 64
    return A[:, keep], B[:, keep], logv[keep], [k for k, m in zip(keys, keep) if m]


def chi_stat(A, B):
    se2 = A.var(0, ddof=1) / len(A) + B.var(0, ddof=1) / len(B)
    ok = se2 > 0
    return float(np.sum((A.mean(0)[ok] - B.mean(0)[ok]) ** 2 / se2[ok]))


def ks_stat(A, B, logv):
    o = np.argsort(logv)
    ca, cb = np.cumsum(A.sum(0)[o]), np.cumsum(B.sum(0)[o])
    return float(np.max(np.abs(ca / ca[-1] - cb / cb[-1])))


def permutation_p(A, B, logv, nperm=2000, seed=0):
    rng = np.random.default_rng(seed)
    X, na = np.vstack([A, B]), len(A)
    c0, k0 = chi_stat(A, B), ks_stat(A, B, logv)
    cc = kc = 0
    for _ in range(nperm):
        p = rng.permutation(len(X))
        a, b = X[p[:na]], X[p[na:]]
        cc += chi_stat(a, b) >= c0
        kc += ks_stat(a, b, logv) >= k0
    return (cc + 1) / (nperm + 1), (kc + 1) / (nperm + 1)


def test_single_type_agrees_in_distribution(oracle_lib):
    d, R = load("reference_single_type.json")
    w = cfg.small()
    w.types = [tuple(t) for t in d["types"]]
    O = oracle_runs(oracle_lib, w, len(R), 9000)
    A, B, logv, _ = matrices(R, O)
    p_chi, p_ks = permutation_p(A, B, logv)
    assert p_chi > 0.01 and p_ks > 0.01, (p_chi, p_ks)
    # totals per run: means within 3 standard errors
    ta, tb = A.sum(1), B.sum(1)
    assert abs(ta.mean() - tb.mean()) < 3 * np.sqrt(ta.var(ddof=1) / len(ta) + tb.var(ddof=1) / len(tb))


def test_two_types_show_the_reference_type_timer_coupling(oracle_lib):
    d, R = load("reference_small.json")
    w = cfg.small()
    O = oracle_runs(oracle_lib, w, len(R), 9000)
    A, B, logv, keys = matrices(R, O)
    p_chi, _ = permutation_p(A, B, logv, nperm=200)
    assert p_chi < 0.01
    # the root generation: values equal to a nonzero bin's own value
    roots = {"%.10g" % v for v, f in w.bins if f}
    idx = [i for i, k in enumerate(keys) if k in roots]
    ga, gb = A[:, idx].sum(1), B[:, idx].sum(1)
    se = np.sqrt(ga.var(ddof=1) / len(ga) + gb.var(ddof=1) / len(gb))
    assert gb.mean() - ga.mean() > 10 * se


def oracle_typed_runs(oracle_lib, w, n, base):
    out = []
    for k in range(n):
        o = oracle_lib.simulate(w.bins, w.types, w.t_max, w.phi, seed=base + k)
        out.append({"%.10g" % v: p.astype(float) for v, p in zip(o.values, o.per_type) if p.sum()})
    return out


def test_shared_timers_isolate_the_type_coupling(oracle_lib):
    d, R = load("reference_same_timer.json")
    assert d["binary"] == "procell_ref_sm100"
    w = cfg.small()
    w.types = [tuple(t) for t in d["types"]]
    assert w.types[0][1:] == w.types[1][1:]
    O = oracle_runs(oracle_lib, w, len(R), 9000)
    A, B, logv, keys = matrices(R, O)
    # totals: the type cannot change any division time, and the histograms agree
    p_chi, p_ks = permutation_p(A, B, logv)
    assert p_chi > 0.01 and p_ks > 0.01, (p_chi, p_ks)
    ta, tb = A.sum(1), B.sum(1)
    assert abs(ta.mean() - tb.mean()) < 3 * np.sqrt(ta.var(ddof=1) / len(ta) + tb.var(ddof=1) / len(tb))
    # per-type columns: generation-0 leaves (values equal to a nonzero bin's own value)
    vals = ["%.10g" % float.fromhex(v) for v in d["values"]]
    roots = {"%.10g" % v for v, f in w.bins if f}
    g0 = np.array([v in roots for v in vals])
    ref_pt = np.array(d["per_type"], float)           # [run][value][type]
    ref_g0 = ref_pt[:, g0, :].sum(axis=1)             # [run][type]
    OT = oracle_typed_runs(oracle_lib, w, len(R), 9000)
    or_g0 = np.array([sum((p for k, p in r.items() if k in roots), np.zeros(2)) for r in OT])
    # the same number of roots out of time at generation 0 ...
    sa, sb = ref_g0.sum(1), or_g0.sum(1)
    assert abs(sa.mean() - sb.mean()) < 3 * np.sqrt(sa.var(ddof=1) / len(sa) + sb.var(ddof=1) / len(sb))
    # ... but in the reference all of type 0: no type-1 root ever stays undivided past t_max
    assert ref_g0[:, 1].sum() == 0 and ref_g0[:, 0].mean() > 50
    assert or_g0[:, 1].mean() > 25 and or_g0[:, 0].mean() > 25
    # and over all leaves, type 0 holds more than its ratio's share in the reference only
    fa = ref_pt[:, :, 0].sum(1) / ref_pt.sum(axis=(1, 2))
    fb = np.array([sum(p[0] for p in r.values()) / sum(p.sum() for p in r.values()) for r in OT])
    se = np.sqrt(fa.var(ddof=1) / len(fa) + fb.var(ddof=1) / len(fb))
    assert fa.mean() - fb.mean() > 10 * se and abs(fb.mean() - 0.53) < 0.01


def test_medium_shared_timers_agree_without_lost_subtrees(oracle_lib):
    d, R = load("reference_medium_t150_same_timer.json")
    assert d["binary"] == "procell_ref_sm100" and len(R) == 16
    w = cfg.medium()
    w.t_max = d["t_max"]
    w.types = [tuple(t) for t in d["types"]]
    O = oracle_runs(oracle_lib, w, len(R), 9000)
    A, B, logv, _ = matrices(R, O)
    ta, tb = A.sum(1), B.sum(1)
    se = np.sqrt(ta.var(ddof=1) / len(ta) + tb.var(ddof=1) / len(tb))
    assert abs(ta.mean() - tb.mean()) < 3 * se, (ta.mean(), tb.mean(), se)
    p_chi, _ = permutation_p(A, B, logv, nperm=500)
    assert p_chi > 0.01, p_chi
    assert ks_stat(A, B, logv) < 1e-3
