"""Log level (reference: utils/set_log_level.py:5-18), on Python logging."""
import logging
import sys

_LEVELS = {"TRACE": 5, "DEBUG": 10, "INFO": 20, "SUCCESS": 25, "WARNING": 30, "ERROR": 40, "CRITICAL": 50}


def set_log_level(log_level: str):
    logger = logging.getLogger("torchquad_gb300")
    for h in list(logger.handlers):
        logger.removeHandler(h)
    h = logging.StreamHandler(sys.stderr)
    h.setFormatter(logging.Formatter("%(asctime)s|TQ-%(levelname)s| %(message)s", "%H:%M:%S"))
    logger.addHandler(h)
    logger.setLevel(_LEVELS.get(log_level.upper(), 30))
