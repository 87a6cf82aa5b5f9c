"""Package logger (replaces jax_fem/logger_setup.py:4-28; no banner on import)."""
import logging

logger = logging.getLogger("jax_fem_gb300")
if not logger.handlers:
    _h = logging.StreamHandler()
    _h.setFormatter(logging.Formatter("[%(asctime)s][%(levelname)s] %(name)s: %(message)s", "%H:%M:%S"))
    logger.addHandler(_h)
    logger.setLevel(logging.WARNING)
    logger.propagate = False


def set_level(level):
    logger.setLevel(level)
