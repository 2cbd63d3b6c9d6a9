"""python/FLUE/gluonCalc/su3matrixops.py:1-4 over the GB300 library."""
from FLUE.compiled import flue_c as fc


def multiplymatmat(left, right):
    return fc.multiplymatmat_c(left, right)


def fixsu3matrix(u_x):
    """Reunitarise a (3,3) complex128 Fortran-contiguous array in place."""
    return fc.fixsu3matrix(u_x)
