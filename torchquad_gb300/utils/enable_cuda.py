"""CUDA check (reference: utils/enable_cuda.py:7-26).  Every kernel of this
package runs on the current CUDA device, so this only verifies the device and
optionally sets the default precision."""
import logging
import warnings

from .set_precision import set_precision

logger = logging.getLogger("torchquad_gb300")


def enable_cuda(data_type="float32"):
    import torch

    if torch.cuda.is_available():
        logger.info("Active CUDA Device: GPU%d", torch.cuda.current_device())
        if data_type is not None:
            set_precision(data_type)
    else:
        msg = (
            "Error enabling CUDA. cuda.is_available() returned False. torchquad_gb300 "
            "has no CPU path; integration calls will raise."
        )
        logger.warning(msg)
        warnings.warn(msg, RuntimeWarning)
