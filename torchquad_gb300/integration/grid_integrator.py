"""GridIntegrator (reference: integration/grid_integrator.py:14-255).

Two execution paths, both on the GPU:

* fused — the integrand is a built-in family (``torchquad_gb300.integrands``):
  one kernel generates every node from its flat index, evaluates the
  integrand and accumulates the weighted sum (no point tensor exists);
* materialised — any vectorised torch callable: a kernel writes the points
  of a chunk in the reference's layout (``[N, dim]``, last dimension
  fastest), the callable runs on them, and a weighted-sum kernel applies the
  tensor-product weights.  Gradients w.r.t. the domain and the integrand's
  tensors flow through torch autograd and the kernel's adjoint
  (``_kernels.WeightedSum``).
"""
from __future__ import annotations

import math

import torch

from .. import _lib as L
from ..integrands import BuiltinIntegrand
from . import _kernels as K
from .base_integrator import BaseIntegrator
from .utils import (
    _assemble_result,
    _setup_integration_domain,
    _split_integrand_values,
    _host_domain_check,
)


def _grid_check(N, dim):
    """IntegrationGrid._check_inputs (integration_grid.py:105-124)."""
    if N < 2:
        raise ValueError("N has to be > 1.")
    if N ** (1.0 / dim) < 2:
        raise ValueError(
            "Cannot create a ",
            dim,
            "-dimensional grid with ",
            N,
            " points. Too few points per dimension.",
        )


def _n_per_dim(N, dim):
    # integration_grid.py:64 — the 1e-8 guards against (4**3)**(1/3) = 3.999...
    return int(N ** (1.0 / dim) + 1e-8)


class _FusedGridFn(torch.autograd.Function):
    """Fused rule with a hand-written adjoint: forward is tq_grid_fused,
    backward is tq_grid_adjoint (value and all gradients in one pass)."""

    @staticmethod
    def forward(ctx, domain, c, b, a, u, integ, fn, dim, n):
        ctx.integ, ctx.fn, ctx.dim, ctx.n = integ, fn, dim, n
        ctx.save_for_backward(domain, c, b, a, u)
        return integ._integrate_fused(fn, dim, n, domain.detach())

    @staticmethod
    def backward(ctx, gout):
        domain, c, b, a, u = ctx.saved_tensors
        integ, fn, dim, n = ctx.integ, ctx.fn, ctx.dim, ctx.n
        gl_nodes, gl_w = integ._gl_tables(n, domain.device)
        _, gdom, gpar = K.grid_adjoint(integ._rule, dim, n, domain.detach(), gl_nodes, gl_w, fn)
        g = gout.detach().to(torch.float64)

        def back(t, grad):
            if t is None or not t.requires_grad:
                return None
            return (g * grad).reshape(t.shape).to(t.device, t.dtype)

        return (back(domain, gdom), back(c, gpar[0]), back(b, gpar[1]), back(a, gpar[2 : 2 + dim]),
                back(u, gpar[2 + dim : 2 + 2 * dim]), None, None, None, None)


class GridIntegrator(BaseIntegrator):
    """Base of the tensor-product rules (Newton-Cotes and Gaussian)."""

    _rule = None  # TQ_RULE_* of the subclass

    def __init__(self):
        super().__init__()

    # ------------------------------------------------------------ public
    def integrate(self, fn, dim, N, integration_domain, backend):
        """Integrate fn over the domain with the composite rule of the
        subclass; returns a 0-d tensor for scalar integrands."""
        if N is None:
            N = self._get_minimal_N(dim)
        domain = self._prepare_domain(dim, N, integration_domain, backend)
        N = self._adjust_N(dim=dim, N=N)
        _grid_check(N, dim)
        n = _n_per_dim(N, dim)
        self._nr_of_fevals = n**dim
        if self._can_fuse(fn, dim, domain):
            return self._integrate_fused(fn, dim, n, domain)
        if self._can_fuse_adjoint(fn, dim):
            return _FusedGridFn.apply(domain, fn.c, fn.b, fn.a, fn.u, self, fn, dim, n)
        return self._integrate_materialised(fn, dim, n, domain)

    def calculate_grid(self, N, integration_domain, disable_integration_domain_check=False):
        """(points [n^dim, dim], h [dim], n) as grid_integrator.py:93-127."""
        from .integration_grid import IntegrationGrid

        dim = integration_domain.shape[0] if isinstance(integration_domain, torch.Tensor) else len(integration_domain)
        N = self._adjust_N(dim=dim, N=N)
        grid = IntegrationGrid(N, integration_domain, None, disable_integration_domain_check, integrator=self)
        return grid.points, grid.h, grid._N

    def calculate_result(self, function_values, dim, n_per_dim, hs, integration_domain):
        """Apply the composite rule to function values of a calculate_grid
        grid (grid_integrator.py:57-91) with the weighted-sum kernel."""
        domain = integration_domain
        values, shape, is_complex = _split_integrand_values(function_values)
        gl_w = self._gl_tables(n_per_dim, domain.device)[1]
        if torch.is_grad_enabled() and domain.requires_grad:
            unit = self._unit_domain(domain)
            out = K.WeightedSum.apply(values, self._rule, dim, n_per_dim, unit, gl_w, 0)
            out = out * self._weight_scale(domain, dim).to(out.dtype)
        else:
            out = K.WeightedSum.apply(values, self._rule, dim, n_per_dim, domain.detach(), gl_w, 0)
        return _assemble_result(out, shape, is_complex)

    @staticmethod
    def _adjust_N(dim, N):
        return N

    def get_jit_compiled_integrate(self, dim, N=None, integration_domain=None, backend=None):
        """Return integrate(fn, integration_domain) with N and dim fixed.

        The reference traces calculate_grid/calculate_result with
        torch.jit.trace (grid_integrator.py:133-255).  Here both steps are
        already single kernels, so the returned function calls them
        directly; the grid size is validated once."""
        if N is None:
            N = self._get_minimal_N(dim)
        self._prepare_domain(dim, N, integration_domain, backend)
        N_adj = self._adjust_N(dim=dim, N=N)
        _grid_check(N_adj, dim)

        def compiled_integrate(fn, integration_domain):
            return self.integrate(fn, dim, N, integration_domain, backend)

        return compiled_integrate

    # ------------------------------------------------------------ helpers
    def _prepare_domain(self, dim, N, integration_domain, backend):
        if integration_domain is not None and not isinstance(integration_domain, torch.Tensor):
            if hasattr(integration_domain, "__len__"):
                _host_domain_check(integration_domain)
        domain = _setup_integration_domain(dim, integration_domain, backend)
        self._check_inputs(dim=dim, N=N, integration_domain=None if not isinstance(integration_domain, torch.Tensor) else domain)
        return domain

    def _result_dtype(self, domain):
        return domain.dtype

    def _gl_tables(self, n, device):
        return None, None

    def _weight_scale(self, domain, dim):
        """prod_k of the domain-dependent factor of the 1-D weights."""
        return torch.prod(domain[:, 1] - domain[:, 0])

    def _unit_domain(self, domain):
        z = torch.zeros_like(domain.detach())
        z[:, 1] = 1.0
        return z

    def _points_from_unit(self, unit_pts, domain):
        a = domain[:, 0]
        return unit_pts * (domain[:, 1] - a) + a

    def _can_fuse(self, fn, dim, domain):
        if not isinstance(fn, BuiltinIntegrand) or fn.dim != dim or dim > L.TQ_MAX_DIM:
            return False
        if torch.is_grad_enabled() and (domain.requires_grad or fn.requires_grad()):
            return False
        return True

    def _can_fuse_adjoint(self, fn, dim):
        """Built-in integrand whose gradient the adjoint kernel computes."""
        return (isinstance(fn, BuiltinIntegrand) and fn.dim == dim and dim <= 8
                and getattr(self, "_rescales_nodes", True))

    def _integrate_fused(self, fn, dim, n, domain):
        gl_nodes, gl_w = self._gl_tables(n, domain.device)
        return K.grid_fused(self._rule, dim, n, domain, gl_nodes, gl_w, fn, self._result_dtype(domain))

    def _integrate_materialised(self, fn, dim, n, domain):
        total = n**dim
        gl_nodes, gl_w = self._gl_tables(n, domain.device)
        pdtype = torch.float64 if self._rule == L.TQ_RULE_GAUSS else domain.dtype
        grad = torch.is_grad_enabled() and domain.requires_grad
        if grad:
            # Differentiable in the bounds, as utils.py:36-52 / gaussian.py:
            # 159-162: unit-domain nodes, scaled with torch ops, unit weights
            # times the product of the per-dimension widths.
            unit = self._unit_domain(domain)
            pts = K.grid_points(self._rule, dim, n, unit, gl_nodes, 0, total, pdtype)
            pts = self._points_from_unit(pts, domain)
            vals, _ = self.evaluate_integrand(fn, pts)
            values, shape, is_complex = _split_integrand_values(vals)
            out = K.WeightedSum.apply(values, self._rule, dim, n, unit, gl_w, 0)
            out = out * self._weight_scale(domain, dim).to(out.dtype)
            return _assemble_result(out, shape, is_complex)

        chunk = K.chunk_points(total, dim, torch.finfo(pdtype).bits // 8)
        if torch.is_grad_enabled() and chunk < total:
            chunk = total  # one autograd graph, like the reference
        acc = None
        outs = []
        shape = is_complex = None
        for start in range(0, total, chunk):
            count = min(chunk, total - start)
            pts = K.grid_points(self._rule, dim, n, domain, gl_nodes, start, count, pdtype)
            vals, _ = self.evaluate_integrand(fn, pts)
            values, shape, is_complex = _split_integrand_values(vals)
            if values.requires_grad and torch.is_grad_enabled():
                outs.append(K.WeightedSum.apply(values, self._rule, dim, n, domain, gl_w, start))
                continue
            if acc is None:
                acc = torch.zeros((2 * values.shape[1],), dtype=torch.float64, device=domain.device)
            K.weighted_sum_into(acc, self._rule, dim, n, domain, gl_w, start, values)
        if outs:
            out = outs[0]
            for o in outs[1:]:
                out = out + o
        else:
            out_dtype = torch.promote_types(values.dtype, self._result_dtype(domain))
            out = K.finalize(acc, self._rule, dim, domain, total, values.shape[1], out_dtype)
        return _assemble_result(out, shape, is_complex)
