"""Default floating-point precision (reference: utils/set_precision.py:18-89)."""
import logging
import os
import sys

import torch

logger = logging.getLogger("torchquad_gb300")


def _get_precision(backend):
    """The configured default precision name for ``backend`` or None."""
    return os.environ.get(f"TORCHQUAD_DTYPE_{backend.upper()}", None)


def set_precision(data_type="float32", backend="torch"):
    """Set torch's default floating point dtype ("float32"/"float64"; "float"
    and "double" are accepted).  Integration domains given as lists use it.
    Only the torch backend exists in this package."""
    data_type = {"float": "float32", "double": "float64"}.get(data_type.lower(), data_type)
    if data_type not in ["float32", "float64"]:
        msg = (
            f'Invalid data type "{data_type}". Only float32 and float64 are supported. '
            "Setting the data type to float32."
        )
        logger.error(msg)
        print(f"ERROR: {msg}", file=sys.stderr)
        data_type = "float32"
    if backend != "torch":
        msg = f"Changing the data type is not supported for backend {backend}"
        logger.error(msg)
        print(f"ERROR: {msg}", file=sys.stderr)
        return
    torch.set_default_dtype({"float32": torch.float32, "float64": torch.float64}[data_type])
    os.environ["TORCHQUAD_DTYPE_TORCH"] = data_type
