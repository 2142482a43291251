"""The ``pyop2`` logger (pyop2/logger.py:39-93)."""
import logging

logger = logging.getLogger("pyop2")
if not logger.handlers:
    _h = logging.StreamHandler()
    _h.setFormatter(logging.Formatter("%(name)s:%(levelname)s %(message)s"))
    logger.addHandler(_h)

debug = logger.debug
info = logger.info
warning = logger.warning
error = logger.error
critical = logger.critical


def set_log_level(level):
    """Set the log level of the ``pyop2`` logger."""
    logger.setLevel(level)
