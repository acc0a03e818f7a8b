"""Smoothed, differentiable form (pc_smooth_*) and its torch.autograd.Function.

    from procell import Engine
    from procell.smooth import Smooth, expected_counts
    eng = Engine()
    sm = Smooth(eng, bins, n_types=3, t_max=168, phi=None, h=0.5, paths=4, seed=1)
    params = torch.tensor(..., dtype=torch.float64, device="cuda", requires_grad=True)  # [C, K, 3]
    E = expected_counts(sm, params)        # [C, n_values]: expected histogram per candidate
    loss = ((torch.log1p(E) - torch.log1p(target)) ** 2).sum()
    loss.backward()                        # params.grad from the hand-written adjoint kernel

The forward and the adjoint run in libprocell (sm_103a kernels) on the current torch
stream; torch only holds the device arrays.
"""
from __future__ import annotations

import ctypes

import numpy as np
import torch

from . import _lib


class Smooth:
    """A prepared input (bins, t_max, phi, smoothing h, lineages per initial cell, seed)."""

    def __init__(self, engine, bins, n_types, t_max, phi=None, h=0.5, paths=1, seed=0):
        self.engine = engine
        L = engine.L
        b = _lib.bins_numpy(bins)
        h_ = ctypes.c_void_p()
        engine._check(L.pc_smooth_create(engine.ctx, b.ctypes.data_as(ctypes.POINTER(_lib.Bin)), len(b),
                                         int(n_types), float(t_max), 0.0 if phi is None else float(phi),
                                         float(h), int(paths), int(seed), ctypes.byref(h_)))
        self.handle = h_
        nv, nt, nc = ctypes.c_uint64(), ctypes.c_uint32(), ctypes.c_uint64()
        L.pc_smooth_info(self.handle, ctypes.byref(nv), ctypes.byref(nt), ctypes.byref(nc))
        self.n_values, self.n_types, self.n_cells = int(nv.value), int(nt.value), int(nc.value)
        vals = np.zeros(max(1, self.n_values), np.float64)
        L.pc_smooth_values(self.handle, vals.ctypes.data_as(ctypes.POINTER(ctypes.c_double)))
        self.values = vals[:self.n_values]

    def _bind_stream(self):
        self.engine.set_stream(torch.cuda.current_stream().cuda_stream)

    def forward(self, params: torch.Tensor) -> torch.Tensor:
        p = params.detach().to(torch.float64).contiguous()
        assert p.is_cuda and p.dim() == 3 and p.shape[1] == self.n_types and p.shape[2] == 3
        out = torch.empty(p.shape[0], self.n_values, dtype=torch.float64, device=p.device)
        self._bind_stream()
        self.engine._check(self.engine.L.pc_smooth_forward(self.engine.ctx, self.handle, ctypes.c_void_p(p.data_ptr()),
                                                           p.shape[0], ctypes.c_void_p(out.data_ptr())))
        return out

    def backward(self, params: torch.Tensor, grad_expected: torch.Tensor) -> torch.Tensor:
        p = params.detach().to(torch.float64).contiguous()
        g = grad_expected.detach().to(torch.float64).contiguous()
        out = torch.empty_like(p)
        self._bind_stream()
        self.engine._check(self.engine.L.pc_smooth_backward(self.engine.ctx, self.handle, ctypes.c_void_p(p.data_ptr()),
                                                            p.shape[0], ctypes.c_void_p(g.data_ptr()),
                                                            ctypes.c_void_p(out.data_ptr())))
        return out

    def jacobian(self, params: torch.Tensor):
        """(expected [C, n_values], jacobian [C, n_values, n_types, 3]) in one pass:
        jacobian[c, v, k] = d expected[c, v] / d (ratio, mean, sd) of type k."""
        p = params.detach().to(torch.float64).contiguous()
        assert p.is_cuda and p.dim() == 3 and p.shape[1] == self.n_types and p.shape[2] == 3
        E = torch.empty(p.shape[0], self.n_values, dtype=torch.float64, device=p.device)
        J = torch.empty(p.shape[0], self.n_values, self.n_types, 3, dtype=torch.float64, device=p.device)
        self._bind_stream()
        self.engine._check(self.engine.L.pc_smooth_jacobian(self.engine.ctx, self.handle, ctypes.c_void_p(p.data_ptr()),
                                                            p.shape[0], ctypes.c_void_p(E.data_ptr()),
                                                            ctypes.c_void_p(J.data_ptr())))
        return E, J

    def gauss_newton(self, params: torch.Tensor, target: torch.Tensor):
        """(loss [C], jtj [C, P, P], jtr [C, P]) of sum_v (log1p(E_v) - log1p(target_v))^2,
        P = 3 n_types in the order of params' last two dimensions (type, parameter)."""
        p = params.detach().to(torch.float64).contiguous()
        t = target.detach().to(torch.float64).contiguous()
        assert p.is_cuda and p.dim() == 3 and p.shape[1] == self.n_types and p.shape[2] == 3
        assert t.is_cuda and t.numel() == self.n_values
        C, P = p.shape[0], 3 * self.n_types
        loss = torch.empty(C, dtype=torch.float64, device=p.device)
        jtj = torch.empty(C, P, P, dtype=torch.float64, device=p.device)
        jtr = torch.empty(C, P, dtype=torch.float64, device=p.device)
        self._bind_stream()
        V = ctypes.c_void_p
        self.engine._check(self.engine.L.pc_smooth_gauss_newton(
            self.engine.ctx, self.handle, V(p.data_ptr()), C, V(t.data_ptr()), V(loss.data_ptr()),
            V(jtj.data_ptr()), V(jtr.data_ptr())))
        return loss, jtj, jtr

    def sync(self):
        self.engine._check(self.engine.L.pc_smooth_sync(self.engine.ctx))

    def close(self):
        if getattr(self, "handle", None):
            self.engine.L.pc_smooth_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class ExpectedCounts(torch.autograd.Function):
    """params [C, K, 3] (ratio, mean, sd per type) -> expected counts [C, n_values]."""

    @staticmethod
    def forward(ctx, params, smooth):
        ctx.smooth = smooth
        ctx.save_for_backward(params)
        return smooth.forward(params)

    @staticmethod
    def backward(ctx, grad_out):
        (params,) = ctx.saved_tensors
        return ctx.smooth.backward(params, grad_out), None


def expected_counts(smooth: Smooth, params: torch.Tensor) -> torch.Tensor:
    return ExpectedCounts.apply(params, smooth)
