"""Seeded synthetic workloads for the proliferation path.

The reference ships no data sets or benchmarks; these generators produce inputs with
the shapes and value distributions of the four plain/batched workloads and the
calibration workload the engine is measured on. Every value is a float64 that
round-trips exactly through the `%.17g` text the writers below emit.

* small   64 bins, fluorescence log-uniform on [1, 1e4], frequency Poisson(150),
          types (0.53, 48.33, 21.6) and (0.47, 86.3, 26.8), t_max 168,
          phi = the minimum nonzero bin value.
* medium  1024 bins, log-uniform on [1, 1e5], Poisson(1000), types 0.30/40/12,
          0.30/60/18, 0.22/90/27 and a quiescent 0.18/-1/-1, t_max 336, phi 4,
          per-type tracking on.
* large   4096 bins, log-uniform on [1, 1e6], Poisson(2500), five types with means
          uniform on [30, 60], sd = 0.3 x mean, Dirichlet(1) ratios, t_max 336, phi 1.
* batched 4096 independent instances: bins uniform on {32..1024}, initial cells
          log-uniform on [1e3, 1e6] spread over the bins, fluorescence log-uniform on
          [1, 1e4], 1-4 proliferating types (mean U[20,120], sd U[0.1,0.4] x mean,
          Dirichlet(1) ratios) plus a quiescent type with probability 0.2,
          t_max U[48, 336], phi = minimum nonzero bin value.
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np


@dataclass
class Workload:
    name: str
    bins: list            # [(value, freq)] in file order
    types: list           # [(ratio, mean, sd)] in file order
    t_max: float
    phi: float | None     # None: the reference's automatic threshold
    track_ratio: bool = False
    seed: int = 0         # engine seed (the Philox key)
    meta: dict = field(default_factory=dict)

    @property
    def roots(self) -> int:
        return int(sum(int(f) for _, f in self.bins))


def _ratios_sum_to_one(r: np.ndarray) -> list:
    """Normalise so that the sequential float64 sum is within 1e-8 of 1 (the
    reference's check, src/io/parser.cu:46-66)."""
    r = np.asarray(r, dtype=np.float64)
    r = r / r.sum()
    out = [float(x) for x in r]
    s = 0.0
    for x in out:
        s += x
    assert abs(1.0 - s) <= 1e-8, s
    return out


def _loguniform(rng, lo, hi, n):
    return np.exp(rng.uniform(np.log(lo), np.log(hi), n))


def small(seed: int = 11) -> Workload:
    rng = np.random.default_rng(seed)
    v = _loguniform(rng, 1.0, 1e4, 64)
    f = rng.poisson(150, 64)
    bins = [(float(a), int(b)) for a, b in zip(v, f)]
    phi = float(min(a for a, b in bins if b > 0))
    types = [(0.53, 48.33, 21.6), (0.47, 86.3, 26.8)]
    return Workload("small", bins, types, 168.0, phi, False, seed=seed)


def medium(seed: int = 12) -> Workload:
    rng = np.random.default_rng(seed)
    v = _loguniform(rng, 1.0, 1e5, 1024)
    f = rng.poisson(1000, 1024)
    bins = [(float(a), int(b)) for a, b in zip(v, f)]
    types = [(0.30, 40.0, 12.0), (0.30, 60.0, 18.0), (0.22, 90.0, 27.0), (0.18, -1.0, -1.0)]
    return Workload("medium", bins, types, 336.0, 4.0, True, seed=seed)


def large(seed: int = 13) -> Workload:
    rng = np.random.default_rng(seed)
    v = _loguniform(rng, 1.0, 1e6, 4096)
    f = rng.poisson(2500, 4096)
    bins = [(float(a), int(b)) for a, b in zip(v, f)]
    means = rng.uniform(30.0, 60.0, 5)
    ratios = _ratios_sum_to_one(rng.dirichlet(np.ones(5)))
    types = [(r, float(m), float(0.3 * m)) for r, m in zip(ratios, means)]
    return Workload("large", bins, types, 336.0, 1.0, False, seed=seed)


def batched(n_instances: int = 4096, seed: int = 14, fluor_range=(1.0, 1e4)) -> list:
    rng = np.random.default_rng(seed)
    out = []
    for i in range(n_instances):
        nb = int(rng.integers(32, 1025))
        roots = int(round(float(_loguniform(rng, 1e3, 1e6, 1)[0])))
        v = _loguniform(rng, fluor_range[0], fluor_range[1], nb)
        w = rng.dirichlet(np.ones(nb))
        f = rng.multinomial(roots, w)
        bins = [(float(a), int(b)) for a, b in zip(v, f)]
        nt = int(rng.integers(1, 5))
        quiescent = bool(rng.random() < 0.2)
        k = nt + (1 if quiescent else 0)
        ratios = _ratios_sum_to_one(rng.dirichlet(np.ones(k)))
        types = []
        for j in range(nt):
            m = float(rng.uniform(20.0, 120.0))
            types.append((ratios[j], m, float(rng.uniform(0.1, 0.4) * m)))
        if quiescent:
            types.append((ratios[-1], -1.0, -1.0))
        nz = [a for a, b in bins if b > 0]
        phi = float(min(nz)) if nz else 1.0
        t_max = float(rng.uniform(48.0, 336.0))
        out.append(Workload(f"batched[{i}]", bins, types, t_max, phi, False,
                            seed=seed * 100003 + i))
    return out


def by_name(name: str) -> Workload:
    return {"small": small, "medium": medium, "large": large}[name]()


def write_histogram(path: str, bins) -> None:
    with open(path, "w") as fh:
        for v, f in bins:
            fh.write("%.17g %d\n" % (v, int(f)))


def write_types(path: str, types) -> None:
    with open(path, "w") as fh:
        for r, m, s in types:
            fh.write("%.17g %.17g %.17g\n" % (r, m, s))
