"""MonteCarlo (reference: integration/monte_carlo.py:14-225)."""
from __future__ import annotations

import torch

from .. import _lib as L
from ..integrands import BuiltinIntegrand
from . import _kernels as K
from .base_integrator import BaseIntegrator
from .rng import RNG
from .utils import _assemble_result, _setup_integration_domain, _split_integrand_values


class MonteCarlo(BaseIntegrator):
    """Plain Monte Carlo: V / N * sum f(x_i), x_i uniform in the domain."""

    def __init__(self):
        super().__init__()

    def integrate(self, fn, dim, N=1000, integration_domain=None, seed=None, rng=None, backend=None):
        """Integrate fn with N uniform samples; ``seed`` or an initialised
        ``rng`` (anything with ``uniform(size, dtype)``) selects the draws."""
        self._check_inputs(dim=dim, N=N, integration_domain=integration_domain)
        domain = _setup_integration_domain(dim, integration_domain, backend)
        if rng is None:
            rng = RNG(backend="torch", seed=seed)
        elif seed is not None:
            raise ValueError("seed and rng cannot both be passed")
        if self._can_fuse(fn, dim, domain, rng):
            offset = rng.reserve(N * dim, domain.dtype)
            self._nr_of_fevals = N
            return K.mc_fused(dim, N, domain, fn, rng.seed, rng.stream_id, offset)
        sample_points = self.calculate_sample_points(N, domain, seed=None, rng=rng)
        function_values, self._nr_of_fevals = self.evaluate_integrand(fn, sample_points)
        return self.calculate_result(function_values, domain)

    @staticmethod
    def _can_fuse(fn, dim, domain, rng):
        return (
            isinstance(fn, BuiltinIntegrand)
            and type(rng) is RNG
            and fn.dim == dim
            and dim <= L.TQ_MAX_DIM
            and not (torch.is_grad_enabled() and (domain.requires_grad or fn.requires_grad()))
        )

    def calculate_result(self, function_values, integration_domain):
        """V * sum(f) / N (monte_carlo.py:60-82) with the reduction kernel."""
        domain = integration_domain
        values, shape, is_complex = _split_integrand_values(function_values)
        n = values.shape[0]
        dim = domain.shape[0]
        if torch.is_grad_enabled() and (values.requires_grad or domain.requires_grad):
            s = K.WeightedSum.apply(values, L.TQ_RULE_MC, dim, 1, domain.detach(), None, 0)
            volume = torch.prod(domain[:, 1] - domain[:, 0])
            out = volume.to(s.dtype) * s / n
        else:
            acc = torch.zeros((2 * values.shape[1],), dtype=torch.float64, device=values.device)
            K.weighted_sum_into(acc, L.TQ_RULE_MC, dim, 1, domain, None, 0, values)
            out_dtype = torch.promote_types(values.dtype, domain.dtype)
            out = K.finalize(acc, L.TQ_RULE_MC, dim, domain, n, values.shape[1], out_dtype)
        return _assemble_result(out, shape, is_complex)

    def calculate_sample_points(self, N, integration_domain, seed=None, rng=None):
        """Uniform points in the domain: u * (b - a) + a (monte_carlo.py:84-106)."""
        if rng is None:
            rng = RNG(backend="torch", seed=seed)
        elif seed is not None:
            raise ValueError("seed and rng cannot both be passed")
        dim = integration_domain.shape[0]
        domain_starts = integration_domain[:, 0]
        domain_sizes = integration_domain[:, 1] - domain_starts
        u = rng.uniform(size=[N, dim], dtype=domain_sizes.dtype)
        if not isinstance(u, torch.Tensor):
            u = torch.as_tensor(u)
        u = u.to(domain_sizes.device)
        return u * domain_sizes + domain_starts

    def get_jit_compiled_integrate(self, dim, N=1000, integration_domain=None, seed=None, backend=None):
        """integrate(fn, integration_domain) with dim, N and the RNG stream
        fixed (monte_carlo.py:108-225); each call draws fresh numbers."""
        rng = RNG(backend="torch", seed=seed)

        def compiled_integrate(fn, integration_domain):
            return self.integrate(fn, dim, N, integration_domain, rng=rng, backend=backend)

        return compiled_integrate
