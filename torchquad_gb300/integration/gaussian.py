"""Gaussian and GaussLegendre (reference: integration/gaussian.py:6-162).

Roots and weights come from ``numpy.polynomial.legendre.leggauss`` on the
host in fp64, cached per N as the reference does (:110-129), and are
uploaded once per device into a cached fp64 table that the kernels read.
Nodes are ``(b-a)/2 * r + (a+b)/2`` computed in fp64 (the reference promotes
to the fp64 roots), so results are fp64 whatever the domain dtype, as in the
reference.

A subclass that overrides ``_resize_roots``, ``_apply_composite_rule`` or
``_grid_func`` (custom Gaussian rules) runs the reference's algorithm with
torch operations on the device instead of the fused kernel.
"""
from __future__ import annotations

import numpy
import torch

from .. import _lib as L
from .grid_integrator import GridIntegrator


# Gauss-Legendre roots/weights and their device copies, shared by instances
# that use numpy's leggauss (a pure function of n).
_LEGGAUSS = {}
_GL_DEVICE = {}


def _node_count(N):
    """N as a Python int: ints as they are, 0-d tensors and numpy scalars
    through ``item()`` (the reference's rule, gaussian.py:120-124)."""
    if isinstance(N, int):
        return N
    if hasattr(N, "item"):
        return N.item()
    raise NotImplementedError(f"N {N} is not an int and lacks an `item` method")


class Gaussian(GridIntegrator):
    """Gauss-Legendre on [-1, 1] by default; base of custom Gaussian rules.

    As in the reference, the base class does not move the roots into the
    domain (``_resize_roots`` is the identity) but scales each dimension's
    sum by 0.5 * (b - a)."""

    _rule = L.TQ_RULE_GAUSS
    _rescales_nodes = False

    def __init__(self):
        super().__init__()
        self.name = "Gauss-Legendre"
        self._root_fn = numpy.polynomial.legendre.leggauss
        self._root_args = ()
        self._cache = {}
        self._dev_cache = {}

    def integrate(self, fn, dim, N=8, integration_domain=None, backend=None):
        """Integrate fn with a tensor-product Gaussian rule of about N points."""
        if self._is_custom():
            return self._integrate_generic(fn, dim, N, integration_domain, backend)
        return super().integrate(fn, dim, N, integration_domain, backend)

    # ---- reference helper API (gaussian.py:44-129)
    def _weights(self, N, dim, backend=None, requires_grad=False):
        w = torch.as_tensor(self._cached_points_and_weights(N)[1], device=L.require_cuda())
        w.requires_grad = requires_grad
        return torch.prod(torch.stack(list(torch.meshgrid(*([w] * dim), indexing="ij")), dim=0), dim=0).ravel()

    def _roots(self, N, backend=None, requires_grad=False):
        roots = torch.as_tensor(self._cached_points_and_weights(N)[0], device=L.require_cuda())
        if requires_grad:
            roots.requires_grad = True
        return roots

    @property
    def _grid_func(self):
        def f(integration_domain, N, requires_grad=False, backend=None):
            return self._resize_roots(integration_domain, self._roots(N, backend, requires_grad))

        return f

    def _resize_roots(self, integration_domain, roots):
        return roots

    def _cached_points_and_weights(self, N):
        """(roots, weights) of this rule for N nodes per dimension, cached
        under (N, *_root_args) as the reference's subclasses expect
        (gaussian.py:109-128)."""
        key = (_node_count(N), *self._root_args)
        found = self._cache.get(key)
        if found is None:
            found = self._cache[key] = self._compute_roots(key)
        return found

    def _compute_roots(self, key):
        if self._root_fn is not numpy.polynomial.legendre.leggauss:
            return self._root_fn(*key)
        if key[0] > 20000:
            raise ValueError(
                f"{key[0]} Gauss-Legendre nodes per dimension: numpy.polynomial.legendre.leggauss "
                "builds an n x n matrix; use at most 20000")
        # leggauss is a pure function of n: one copy serves every instance
        # (the reference keeps one per instance)
        if key not in _LEGGAUSS:
            _LEGGAUSS[key] = self._root_fn(*key)
        return _LEGGAUSS[key]

    @staticmethod
    def _apply_composite_rule(cur_dim_areas, dim, hs, domain):
        """Collapse the trailing ``dim`` node axes: the plain sum of the
        weighted values times the product of the half-widths (b - a) / 2
        (the factor the roots on [-1, 1] leave out; gaussian.py:130-143
        applies it one axis at a time)."""
        node_axes = tuple(range(cur_dim_areas.dim() - dim, cur_dim_areas.dim()))
        half_widths = torch.stack([0.5 * (domain[d][1] - domain[d][0]) for d in range(dim)])
        return torch.prod(half_widths) * torch.sum(cur_dim_areas, dim=node_axes)

    # ---- kernel plumbing
    def _gl_tables(self, n, device):
        key = (n, self._root_args, str(device))
        shared = self._root_fn is numpy.polynomial.legendre.leggauss
        t = self._dev_cache.get(key)
        if t is None and shared:
            t = _GL_DEVICE.get(key)
        if t is None:
            r, w = self._cached_points_and_weights(n)
            t = (
                torch.as_tensor(numpy.asarray(r, dtype=numpy.float64)).to(device),
                torch.as_tensor(numpy.asarray(w, dtype=numpy.float64)).to(device),
            )
            if shared:
                _GL_DEVICE[key] = t
        self._dev_cache[key] = t
        return t

    def _result_dtype(self, domain):
        return torch.float64

    def _unit_domain(self, domain):
        z = torch.empty_like(domain.detach())
        z[:, 0] = -1.0
        z[:, 1] = 1.0
        return z

    def _weight_scale(self, domain, dim):
        return torch.prod(0.5 * (domain[:, 1] - domain[:, 0]))

    def _points_from_unit(self, unit_pts, domain):
        if not self._rescales_nodes:
            return unit_pts
        a, b = domain[:, 0], domain[:, 1]
        return ((b - a) / 2).to(unit_pts.dtype) * unit_pts + ((a + b) / 2).to(unit_pts.dtype)

    def _kernel_domain(self, domain):
        # The base class keeps the roots on [-1, 1]: run the kernels there and
        # scale the result by prod 0.5 (b - a) afterwards.
        return domain if self._rescales_nodes else self._unit_domain(domain)

    def _integrate_fused(self, fn, dim, n, domain):
        out = super()._integrate_fused(fn, dim, n, self._kernel_domain(domain))
        return out if self._rescales_nodes else out * self._weight_scale(domain, dim).to(out.dtype)

    def _integrate_materialised(self, fn, dim, n, domain):
        if self._rescales_nodes or (torch.is_grad_enabled() and domain.requires_grad):
            return super()._integrate_materialised(fn, dim, n, domain)
        out = super()._integrate_materialised(fn, dim, n, self._unit_domain(domain))
        return out * self._weight_scale(domain, dim).to(out.dtype)

    # ---- custom subclasses: the reference algorithm in torch operations
    def _is_custom(self):
        cls = type(self)
        base = GaussLegendre if isinstance(self, GaussLegendre) else Gaussian
        return (
            cls._resize_roots is not base._resize_roots
            or cls._apply_composite_rule is not Gaussian._apply_composite_rule
            or type(self)._grid_func is not Gaussian._grid_func
        )

    def _integrate_generic(self, fn, dim, N, integration_domain, backend):
        from .utils import _assemble_result

        if N is None:
            N = self._get_minimal_N(dim)
        domain = self._prepare_domain(dim, N, integration_domain, backend)
        n = int(N ** (1.0 / dim) + 1e-8)
        grid_1d = [self._grid_func(domain[d], n, domain.requires_grad) for d in range(dim)]
        hs = torch.stack([g[1] - g[0] for g in grid_1d])
        mesh = torch.meshgrid(*grid_1d, indexing="ij")
        points = torch.stack([m.ravel() for m in mesh], dim=1)
        values, num = self.evaluate_integrand(fn, points, weights=self._weights(n, dim))
        self._nr_of_fevals = num
        shape = tuple(values.shape[1:])
        v = values.reshape(num, -1).movedim(0, -1).reshape(-1, *([n] * dim))
        out = self._apply_composite_rule(v, dim, hs, domain)
        return _assemble_result(out.reshape(-1), shape, False) if not values.is_complex() else out.reshape(shape)


class GaussLegendre(Gaussian):
    """Gauss-Legendre quadrature on any domain [a, b]^dim."""

    _rescales_nodes = True

    def __init__(self):
        super().__init__()

    def _resize_roots(self, integration_domain, roots):
        a = integration_domain[0]
        b = integration_domain[1]
        return ((b - a) / 2) * roots + ((a + b) / 2)
