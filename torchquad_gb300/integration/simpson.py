"""Simpson (reference: integration/simpson.py:7-83)."""
import warnings

from .. import _lib as L
from .newton_cotes import NewtonCotes


class Simpson(NewtonCotes):
    """Composite Simpson 1-4-1 rule; needs an odd number >= 3 of points per dimension."""

    _rule = L.TQ_RULE_SIMPSON

    def __init__(self):
        super().__init__()

    def integrate(self, fn, dim, N=None, integration_domain=None, backend=None):
        """Integrate fn with Simpson's rule; N defaults to 3**dim."""
        return super().integrate(fn, dim, N, integration_domain, backend)

    @staticmethod
    def _get_minimal_N(dim):
        return 3**dim

    @staticmethod
    def _adjust_N(dim, N):
        """Odd n >= 3 points per dimension, with the reference's warnings
        (simpson.py:53-83)."""
        n_per_dim = int(N ** (1.0 / dim) + 1e-8)
        if n_per_dim < 3:
            warnings.warn("N per dimension cannot be lower than 3. N per dim will now be changed to 3.")
            N = 3**dim
        elif n_per_dim % 2 != 1:
            warnings.warn(
                "N per dimension cannot be even due to necessary subdivisions. "
                "N per dim will now be changed to the next lower integer, i.e. "
                f"{n_per_dim} -> {n_per_dim - 1}."
            )
            N = (n_per_dim - 1) ** (dim)
        return N
