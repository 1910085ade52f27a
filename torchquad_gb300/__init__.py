"""torchquad_gb300: torchquad's integration hot path on GB300 (sm_103a).

Drop-in names of the reference torchquad package (torch backend only).
Every integration runs in hand-written CUDA kernels behind the C ABI of
``include/torchquad_gb300.h``; there is no CPU fallback.
"""
import os

__version__ = "0.1.0"

from .integration.integration_grid import IntegrationGrid
from .integration.monte_carlo import MonteCarlo
from .integration.trapezoid import Trapezoid
from .integration.simpson import Simpson
from .integration.boole import Boole
from .integration.gaussian import GaussLegendre, Gaussian
from .integration.grid_integrator import GridIntegrator
from .integration.base_integrator import BaseIntegrator
from .integration.rng import RNG
from .integration.vegas import VEGAS
from .integration.vegas_map import VEGASMap
from .integration.vegas_stratification import VEGASStratification
from .integration._kernels import set_materialise_budget

from .utils.set_log_level import set_log_level
from .utils.enable_cuda import enable_cuda
from .utils.set_precision import set_precision
from .utils.set_up_backend import set_up_backend

from . import integrands
from . import batch
from . import serving
from . import vegas_batch
from .vegas_batch import VegasBatch
from .integrands import ExpSum, GaussianPeak, Oscillatory, SumSin, BuiltinIntegrand

__all__ = [
    "__version__",
    "GridIntegrator",
    "BaseIntegrator",
    "IntegrationGrid",
    "MonteCarlo",
    "VEGAS",
    "VEGASMap",
    "VEGASStratification",
    "Trapezoid",
    "Simpson",
    "Boole",
    "GaussLegendre",
    "Gaussian",
    "RNG",
    "enable_cuda",
    "set_precision",
    "set_log_level",
    "set_up_backend",
    "set_materialise_budget",
    "integrands",
    "batch",
    "serving",
    "vegas_batch",
    "VegasBatch",
    "ExpSum",
    "GaussianPeak",
    "Oscillatory",
    "SumSin",
    "BuiltinIntegrand",
]

if os.environ.get("TORCHQUAD_LOG_LEVEL"):
    set_log_level(os.environ["TORCHQUAD_LOG_LEVEL"])
