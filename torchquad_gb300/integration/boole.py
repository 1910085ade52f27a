"""Boole (reference: integration/boole.py:7-84)."""
import warnings

from .. import _lib as L
from .newton_cotes import NewtonCotes


class Boole(NewtonCotes):
    """Composite Boole 7-32-12-32-7 rule; needs n = 4k+1 >= 5 points per dimension."""

    _rule = L.TQ_RULE_BOOLE

    def __init__(self):
        super().__init__()

    def integrate(self, fn, dim, N=None, integration_domain=None, backend=None):
        """Integrate fn with Boole's rule; N defaults to 5**dim."""
        return super().integrate(fn, dim, N, integration_domain, backend)

    @staticmethod
    def _get_minimal_N(dim):
        return 5**dim

    @staticmethod
    def _adjust_N(dim, N):
        """n = 4k+1 >= 5 points per dimension, with the reference's warnings
        (boole.py:55-84)."""
        n_per_dim = int(N ** (1.0 / dim) + 1e-8)
        if n_per_dim < 5:
            warnings.warn("N per dimension cannot be lower than 5. N per dim will now be changed to 5.")
            N = 5**dim
        elif (n_per_dim - 1) % 4 != 0:
            new_n_per_dim = n_per_dim - ((n_per_dim - 1) % 4)
            warnings.warn(
                "N per dimension must be N = 1 + 4n with n a positive integer due to necessary "
                "subdivisions. N per dim will now be changed to the next lower N satisfying this, "
                f"i.e. {n_per_dim} -> {new_n_per_dim}."
            )
            N = (new_n_per_dim) ** (dim)
        return N
