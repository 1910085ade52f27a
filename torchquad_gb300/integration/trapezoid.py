"""Trapezoid (reference: integration/trapezoid.py:6-37)."""
from .. import _lib as L
from .newton_cotes import NewtonCotes


class Trapezoid(NewtonCotes):
    """Composite trapezoidal rule on a tensor-product grid."""

    _rule = L.TQ_RULE_TRAPEZOID

    def __init__(self):
        super().__init__()

    def integrate(self, fn, dim, N=1000, integration_domain=None, backend=None):
        """Integrate fn over integration_domain (default [-1,1]^dim) with
        about N points (int(N**(1/dim)) per dimension)."""
        return super().integrate(fn, dim, N, integration_domain, backend)

    @staticmethod
    def _get_minimal_N(dim):
        return 2**dim
