"""Host-side logic that needs no GPU: N adjustment, input validation and
the RNG's counter bookkeeping, checked against the reference's behaviour."""
import warnings

import numpy as np
import pytest
import torch

import torchquad_gb300 as tq
from torchquad_gb300.integration.base_integrator import BaseIntegrator
from torchquad_gb300.integration.utils import _check_integration_domain, _host_domain_check


def test_simpson_adjust_n_warnings():
    with pytest.warns(UserWarning, match="cannot be lower than 3"):
        assert tq.Simpson._adjust_N(2, 4) == 9
    with pytest.warns(UserWarning, match="cannot be even"):
        assert tq.Simpson._adjust_N(3, 1076890) == 101**3
    with warnings.catch_warnings():
        warnings.simplefilter("error")
        assert tq.Simpson._adjust_N(3, 101**3) == 101**3


def test_boole_adjust_n_warnings():
    with pytest.warns(UserWarning, match="cannot be lower than 5"):
        assert tq.Boole._adjust_N(1, 4) == 5
    with pytest.warns(UserWarning, match="1 \\+ 4n"):
        assert tq.Boole._adjust_N(3, 1000) == 9**3


def test_minimal_n():
    assert tq.Simpson._get_minimal_N(3) == 27
    assert tq.Boole._get_minimal_N(2) == 25


@pytest.mark.parametrize(
    "kwargs",
    [dict(dim=0), dict(N=0), dict(N=2.5), dict(dim=2, integration_domain=[[0, 1]])],
)
def test_check_inputs_errors(kwargs):
    with pytest.raises(ValueError):
        BaseIntegrator._check_inputs(**kwargs)


def test_domain_checks():
    with pytest.raises(ValueError):
        _host_domain_check([[1.0, 0.0]])
    with pytest.raises(ValueError):
        _host_domain_check([[0.0, 1.0, 2.0]])
    with pytest.raises(ValueError):
        _host_domain_check([])
    assert _host_domain_check([[0, 1], [2, 3]]) == 2
    with pytest.raises(ValueError):
        _check_integration_domain(torch.tensor([[1.0, 0.0]]))
    with pytest.raises(ValueError):
        _check_integration_domain(torch.zeros(3))
    assert _check_integration_domain(torch.tensor([[0.0, 1.0]] * 4)) == 4


def test_rng_block_accounting():
    r = tq.RNG(seed=3)
    assert r.reserve(10, torch.float32) == 0
    assert r.offset == 3
    assert r.reserve(3, torch.float64) == 3
    assert r.offset == 5
    with pytest.raises(ValueError):
        tq.RNG(backend="numpy")


def test_non_torch_backend_rejected():
    with pytest.raises(ValueError):
        tq.set_up_backend("jax")


def test_builtin_integrands_match_oracle_on_cpu():
    from oracle import integrands as OI

    x = torch.rand(64, 3, dtype=torch.float64)
    for f in [tq.ExpSum(3, a=[1, 2, 3], b=0.5, c=2.0), tq.GaussianPeak(3, a=[1, 2, 3], u=[0.1, 0.2, 0.3]),
              tq.Oscillatory(3, a=[1, -1, 2], b=0.2), tq.SumSin(3, a=[1, 2, 3], c=0.5)]:
        got = f(x).numpy()
        want = OI.evaluate(f.family, f.params_vector().numpy(), x.numpy())
        assert np.allclose(got, want, rtol=1e-15, atol=0)
