"""Serving: continuous batching.  Every request gives the same result alone
as in a mix of concurrent requests (Simpson and Monte Carlo bit for bit,
VEGAS to rounding), requests are admitted within the HBM budget, and the
served results agree with the per-call API."""
import warnings

import numpy as np
import pytest
import torch

import torchquad_gb300 as tq
from torchquad_gb300.serving import IntegrationRequest, IntegrationServer, poisson_stream

pytestmark = pytest.mark.gpu


def _requests(n=36, seed=7):
    reqs = [r for _, r in poisson_stream(n, rate=1e4, seed=seed, dims=(1, 6), n_range=(1e4, 3e6))]
    for r in reqs:
        r.eps_rel = 0.0  # run to N: identical work alone and in the mix
    return reqs


def _clone(r):
    return IntegrationRequest(r.method, r.integrand, r.N, r.domain, seed=r.seed, eps_rel=r.eps_rel, dtype=r.dtype)


def test_same_result_alone_and_in_the_mix(cuda):
    reqs = _requests()
    alone = []
    with IntegrationServer(max_active=1) as srv:
        for r in reqs:
            f = srv.submit(_clone(r))
            alone.append(f.result(timeout=120))
    mix = []
    with IntegrationServer(max_active=16) as srv:
        futs = [srv.submit(_clone(r)) for r in reqs]
        srv.drain(timeout=300)
        mix = [f.result() for f in futs]
        st = srv.stats()
    assert st["peak_active"] > 1  # requests did overlap
    for r, a, m in zip(reqs, alone, mix):
        if r.method == "vegas":
            assert abs(a - m) <= 1e-9 * max(1e-30, abs(a)), (r.method, a, m)
        else:
            assert a == m, (r.method, a, m)


def test_served_results_match_per_call_api(cuda):
    reqs = _requests(n=12, seed=11)
    with IntegrationServer(max_active=8) as srv:
        futs = [srv.submit(_clone(r)) for r in reqs]
        srv.drain(timeout=300)
        got = [f.result() for f in futs]
    for r, g in zip(reqs, got):
        dom = torch.tensor(r.domain, dtype=r.dtype, device=cuda)
        with warnings.catch_warnings():
            warnings.simplefilter("ignore")
            if r.method == "simpson":
                want = tq.Simpson().integrate(r.integrand, r.dim, N=r.N, integration_domain=dom).item()
                assert abs(g - want) <= 2e-6 * max(1.0, abs(want))
            elif r.method == "montecarlo":
                want = tq.MonteCarlo().integrate(r.integrand, r.dim, N=r.N, integration_domain=dom,
                                                 seed=r.seed).item()
                assert abs(g - want) <= 1e-5 * max(1.0, abs(want))
            else:
                v = tq.VEGAS()
                want = v.integrate(r.integrand, r.dim, N=r.N, integration_domain=dom, seed=r.seed).item()
                assert abs(g - want) <= 1e-5 * max(1e-6, abs(want))


def test_admission_respects_hbm_budget(cuda):
    reqs = [r for r in _requests(n=30, seed=3) if r.method == "vegas"]
    from torchquad_gb300.serving import _footprint

    budget = max(_footprint(r) for r in reqs) * 2
    with IntegrationServer(hbm_budget_bytes=budget, max_active=64) as srv:
        futs = [srv.submit(_clone(r)) for r in reqs]
        srv.drain(timeout=300)
        assert all(np.isfinite(f.result()) for f in futs)
        assert srv.free_bytes == srv.budget
    with pytest.raises(ValueError):
        IntegrationServer(hbm_budget_bytes=1024).submit(_clone(reqs[0]))
