"""Backend selection (reference: utils/set_up_backend.py:8-43).  Only "torch"
is implemented; other backends raise ValueError."""
import os

from .set_precision import set_precision
from .enable_cuda import enable_cuda


def _get_default_backend():
    return os.environ.get("TORCHQUAD_DEFAULT_BACKEND", "torch")


def set_up_backend(backend, data_type=None, torch_enable_cuda=True):
    """Configure the numerical backend; only ``"torch"`` is accepted."""
    if backend != "torch":
        raise ValueError(
            f"Unsupported numerical backend: {backend}. torchquad_gb300 implements the "
            "torch backend only."
        )
    if torch_enable_cuda:
        enable_cuda(data_type=None)
    if data_type is not None:
        set_precision(data_type, backend=backend)
    os.environ["TORCHQUAD_DEFAULT_BACKEND"] = backend
