"""FLUE.gluonCalc: the reference's exports (python/FLUE/gluonCalc/__init__.py:1-4)
plus the wloops observables of the hot path."""
from .su3matrixops import fixsu3matrix, multiplymatmat
from .gluonprop import calc_mom_space_scalarD, scalarGluonProp
from .wloops import (cloverloopmunucoord, genericpath, genplaquette, loop5munucoord, magnetic, magnetic_force,
                     plaquette, polyakov, uzerobar, wmunu, wmunutau)

__all__ = ["multiplymatmat", "calc_mom_space_scalarD", "scalarGluonProp", "fixsu3matrix", "plaquette",
           "genplaquette", "polyakov", "genericpath", "wmunu", "wmunutau", "cloverloopmunucoord", "loop5munucoord",
           "magnetic", "magnetic_force", "uzerobar"]
