"""FLUE.gluonAna (python/FLUE/gluonAna/__init__.py:1-5)."""
from .gpManip import cone_cut, q_average
from .momentum import get_qhat

__all__ = ["q_average", "get_qhat", "cone_cut"]
