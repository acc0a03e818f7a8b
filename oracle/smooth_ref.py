"""CPU restatement of the smoothed (differentiable) form, for tests only.

Test infrastructure, like the rest of oracle/: it checks the sm_103a smoothed-form kernels
and is never part of the product path. It follows the model stated in
cuda-pro-cell_gb300/csrc/pc_smooth.cu independently of that code: the lineage of an initial
cell r, replica m, draws as initial cell r + m * (number of cells): it visits heap nodes
1, 2*1+b_1, ...; node n's standard normal is the oracle's ziggurat draw for child (n & 1) of
parent (n >> 1) (oracle_normals, without the truncation); the initial age U and the path
bits come from the oracle's Philox. Everything
is evaluated in FP64 (the kernels use FP32 log-sigmoids), and the adjoint is obtained by
forward-mode differentiation of the same loop, written separately from the kernel's.

The reference has no smoothed form (the smoothed form is new here); the plain-form pieces it uses
(root age U = tau_1 * U_root, cells_population.cu:124-143; the division rule
proliferation.cu:404-410; the phi cap proliferation.cu:323) are those of the oracle.
"""
from __future__ import annotations

import math

import numpy as np

import oracle

PURPOSE_ROOT = 0x30000000
PURPOSE_PATH = 0x40000000


def _unit53_open_closed(hi, lo):
    m = (int(hi) << 21) | (int(lo) >> 11)
    return float(m + 1) * 1.1102230246251565e-16


def _log_sig(x):
    # log sigmoid(x), log(1 - sigmoid(x))
    L = math.log1p(math.exp(-abs(x)))
    return -(max(-x, 0.0) + L), -(max(x, 0.0) + L)


def prepare(bins, phi):
    """Nonzero bins (value, freq, cap, first root) and the output value set."""
    nz = [(float(v), int(f)) for v, f in bins if int(f) > 0]
    thr = phi if phi else min(v for v, _ in nz)
    out, r0, vals = [], 0, set()
    for v, f in nz:
        cap, x = 0, v
        while x / 2 > thr and cap < 4096:
            cap += 1
            x = x / 2
        out.append((v, f, cap, r0))
        r0 += f
        x = v
        while x >= thr:
            vals.add(x)
            x = x / 2
    return out, sorted(vals), thr


def forward_backward(bins, t_max, phi, h, paths, seed, params, grad_expected=None, with_jacobian=False):
    """Expected counts [C][V] for params [C][K][3], and, with grad_expected [C][V], the
    gradient [C][K][3] of sum(grad_expected * expected). with_jacobian: also the Jacobian
    [C][V][K][3] of the expected counts (returned fourth)."""
    rows, values, thr = prepare(bins, phi)
    ncells = sum(f for _, f, _, _ in rows)
    vindex = {v: i for i, v in enumerate(values)}
    P = np.asarray(params, dtype=np.float64)
    C, K = P.shape[0], P.shape[1]
    E = np.zeros((C, len(values)))
    G = np.zeros((C, K, 3))
    J = np.zeros((C, len(values), K, 3)) if with_jacobian else None
    k0, k1 = seed & 0xFFFFFFFF, seed >> 32
    for (v, f, cap, r0) in rows:
        vi = []
        x = v
        for g in range(cap + 1):
            vi.append(vindex.get(x, -1) if (g > 0 or v >= thr) else -1)
            x = x / 2
        for r in range(r0, r0 + f):
            for m in range(paths):
                vr = r + m * ncells  # replica m draws as initial cell r + m * ncells
                R = oracle.philox([0, 0, vr, PURPOSE_ROOT], [k0, k1])
                U = _unit53_open_closed(R[2], R[3])
                B = oracle.philox([0, 0, vr, PURPOSE_PATH], [k0, k1])
                bits = B[0] | (B[1] << 32)
                nodes, node = [], 1
                for j in range(cap + 1):
                    nodes.append(node)
                    node = 2 * node + ((bits >> j) & 1)
                zs = [float(oracle.normals(seed, vr, n >> 1, 2)[n & 1]) for n in nodes]
                for c in range(C):
                    for k in range(K):
                        ratio, mu, sd = P[c, k]
                        if mu < 0:
                            if vi[0] >= 0:
                                E[c, vi[0]] += ratio / paths
                                if grad_expected is not None:
                                    G[c, k, 0] += grad_expected[c, vi[0]] / paths
                                if J is not None:
                                    J[c, vi[0], k, 0] += 1.0 / paths
                            continue
                        if mu == 0:
                            sd = 0.0
                        S, logp = 0.0, 0.0
                        dS = np.zeros(2)     # d S_j / d(mean, sd)
                        D = np.zeros(2)      # d log(s_1 ... s_{j-1}) / d(mean, sd)
                        for j in range(1, cap + 2):
                            z = zs[j - 1] if mu != 0 else 0.0
                            tau = sd * z + mu
                            if j == 1:
                                S = tau * U + tau
                                dS = np.array([1.0 + U, z * (1.0 + U)])
                            else:
                                S += tau
                                dS = dS + np.array([1.0, z])
                            if mu == 0:
                                dS = np.zeros(2)
                            ls, l1m = _log_sig((t_max - S) / h)
                            w = math.exp(logp + l1m)
                            g = j - 1
                            if vi[g] >= 0:
                                E[c, vi[g]] += ratio * 2.0 ** g * w / paths
                                if J is not None:
                                    s = math.exp(ls)
                                    J[c, vi[g], k, 0] += 2.0 ** g * w / paths
                                    J[c, vi[g], k, 1:] += ratio * 2.0 ** g * w / paths * (D + s / h * dS)
                                if grad_expected is not None:
                                    a = grad_expected[c, vi[g]] * 2.0 ** g * w / paths
                                    G[c, k, 0] += a
                                    s, one_m_s = math.exp(ls), math.exp(l1m)
                                    # d w / d theta = w (D + s / h dS)
                                    G[c, k, 1:] += ratio * a * (D + s / h * dS)
                            D = D - math.exp(l1m) / h * dS
                            logp += ls
                            # the kernels' stopping rule: no later generation can add more
                            # than e^-40 cells
                            if logp < -40.0 - math.log(2.0) * (cap + 1):
                                break
    if with_jacobian:
        return E, G, np.array(values), J
    return E, G, np.array(values)
