"""flue_gb300 -- GB300-native (sm_103a) implementation of FLUE's
gluonic-observable path: plaquettes, Polyakov loop, generic Wilson lines,
W_munu loops, clover and 5-loop F_munu, B^2, u0, their su(3) gradients and the
Wilson flow, behind the reference's Python API (``FLUE.gluonCalc``).

``import flue_gb300 as FLUE`` gives ``FLUE.gluonCalc.<routine>`` with the
reference's names and calling conventions.  All arithmetic runs in the CUDA
library ``libflue_gb300.so`` (C ABI in include/flue_gb300.h).
"""
from . import _lib, field, generate, gluonAna, gluonCalc, gluonProp  # noqa: F401
from .field import GaugeField  # noqa: F401

__version__ = "0.1.0"
__all__ = ["gluonCalc", "gluonProp", "gluonAna", "GaugeField", "field", "generate"]
