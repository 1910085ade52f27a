"""NewtonCotes (reference: integration/newton_cotes.py:4-8)."""
from .grid_integrator import GridIntegrator


class NewtonCotes(GridIntegrator):
    """Abstract base of the closed Newton-Cotes rules."""

    def __init__(self):
        super().__init__()
