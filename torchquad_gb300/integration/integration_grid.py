"""IntegrationGrid (reference: integration/integration_grid.py:19-124).

Stores the tensor-product grid: ``points`` ``[n^dim, dim]`` (last dimension
fastest, as meshgrid(indexing="ij") + stack builds it), the mesh widths ``h``
and ``_N`` points per dimension.  The points are written by the
``tq_grid_points`` kernel; a custom ``grid_func`` produces per-dimension node
arrays that the same node layout is built from.
"""
from __future__ import annotations

from time import perf_counter

import torch

from .. import _lib as L
from . import _kernels as K
from .utils import _check_integration_domain, _setup_integration_domain


def _unit01(domain):
    z = torch.zeros_like(domain.detach())
    z[:, 1] = 1.0
    return z


def grid_func(integration_domain, N, requires_grad=False, backend=None):
    """Equally spaced nodes of one dimension (integration_grid.py:13-16)."""
    a, b = integration_domain[0], integration_domain[1]
    if requires_grad:
        grid = torch.linspace(0.0, 1.0, N, dtype=a.dtype, device=a.device)
        return grid * (b - a) + a
    return torch.linspace(a, b, N, dtype=a.dtype, device=a.device)


class IntegrationGrid:
    points = None
    h = None
    _N = None
    _dim = None
    _runtime = None

    def __init__(self, N, integration_domain, grid_func=None, disable_integration_domain_check=False,
                 integrator=None):
        start = perf_counter()
        self._check_inputs(N, integration_domain, disable_integration_domain_check)
        if not isinstance(integration_domain, torch.Tensor):
            integration_domain = _setup_integration_domain(len(integration_domain), integration_domain, None)
        else:
            if not integration_domain.is_floating_point():
                integration_domain = integration_domain.to(torch.float64)
            if not integration_domain.is_cuda:
                integration_domain = integration_domain.to(L.require_cuda())
        self._dim = integration_domain.shape[0]
        self._N = int(N ** (1.0 / self._dim) + 1e-8)
        requires_grad = bool(integration_domain.requires_grad)

        if grid_func is None:
            rule = getattr(integrator, "_rule", None)
            if rule is None:
                rule = L.TQ_RULE_TRAPEZOID  # every Newton-Cotes rule has these nodes
            gl_nodes = integrator._gl_tables(self._N, integration_domain.device)[0] if integrator else None
            total = self._N**self._dim
            pdtype = torch.float64 if rule == L.TQ_RULE_GAUSS else integration_domain.dtype
            if requires_grad and torch.is_grad_enabled():
                unit = integrator._unit_domain(integration_domain) if integrator else _unit01(integration_domain)
                pts = K.grid_points(rule, self._dim, self._N, unit, gl_nodes, 0, total, pdtype)
                a = integration_domain[:, 0]
                self.points = (integrator._points_from_unit(pts, integration_domain) if integrator
                               else pts * (integration_domain[:, 1] - a) + a)
            else:
                self.points = K.grid_points(rule, self._dim, self._N, integration_domain.detach(),
                                            gl_nodes, 0, total, pdtype)
            self.h = self._h_from_domain(rule, integration_domain, gl_nodes)
        else:
            gf = grid_func if grid_func is not None else globals()["grid_func"]
            grid_1d = [gf(integration_domain[d], self._N, requires_grad=requires_grad) for d in range(self._dim)]
            self.h = torch.stack([g[1] - g[0] for g in grid_1d])
            mesh = torch.meshgrid(*grid_1d, indexing="ij")
            self.points = torch.stack([m.ravel() for m in mesh], dim=1)
        self._runtime = perf_counter() - start

    def _h_from_domain(self, rule, domain, gl_nodes):
        hs = []
        for d in range(self._dim):
            sub = domain[d : d + 1]
            if rule == L.TQ_RULE_GAUSS:
                p = K.grid_points(rule, 1, self._N, sub.detach(), gl_nodes, 0, 2, torch.float64)
                hs.append(p[1, 0] - p[0, 0])
            else:
                a, b = sub[0, 0], sub[0, 1]
                if domain.requires_grad and torch.is_grad_enabled():
                    g = torch.linspace(0.0, 1.0, self._N, dtype=a.dtype, device=a.device)[:2]
                    g = g * (b - a) + a
                else:
                    g = K.grid_points(rule, 1, self._N, sub.detach(), None, 0, 2, domain.dtype)[:, 0]
                hs.append(g[1] - g[0])
        return torch.stack(hs)

    def _check_inputs(self, N, integration_domain, disable_integration_domain_check):
        if disable_integration_domain_check:
            dim = len(integration_domain)
        else:
            dim = _check_integration_domain(integration_domain)
        if N < 2:
            raise ValueError("N has to be > 1.")
        if N ** (1.0 / dim) < 2:
            raise ValueError(
                "Cannot create a ", dim, "-dimensional grid with ", N,
                " points. Too few points per dimension.",
            )
