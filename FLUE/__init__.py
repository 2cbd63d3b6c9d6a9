"""FLUE -- drop-in replacement of the reference's Python package
(python/FLUE/__init__.py:1-4) for the gluonic-observable path, backed by the
GB300 CUDA library ``libflue_gb300.so`` instead of the f2py-wrapped Fortran.

``import FLUE`` gives the same subpackages as the reference:

* ``FLUE.compiled.flue_c`` -- the module f2py builds from
  c_wrapper/FLUE_c.f90 (python/FLUE/compiled/__init__.py:1), here a Python
  module over the library's host-buffer C entry points with f2py's calling
  conventions, widened to the wloops routines of the hot path;
* ``FLUE.gluonCalc`` -- multiplymatmat, calc_mom_space_scalarD,
  scalarGluonProp (python/FLUE/gluonCalc/__init__.py:1-4) and the wloops
  observables (plaquette, polyakov, genericpath, wmunu, clover / 5-loop
  F_munu, magnetic B^2, uzerobar);
* ``FLUE.gluonAna`` -- q_average, get_qhat, cone_cut
  (python/FLUE/gluonAna/__init__.py:1-5).

There is no CPU fallback: every compute call runs on the GPU and fails
loudly when the library or the GPU is missing.
"""
from . import gluonAna, gluonCalc

__all__ = ["gluonAna", "gluonCalc"]
