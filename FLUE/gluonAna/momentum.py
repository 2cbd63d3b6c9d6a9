"""python/FLUE/gluonAna/momentum.py over the GB300 build's flue_c."""
from FLUE.compiled import flue_c as fc


def get_qhat(coord, shape, a=1):
    return fc.get_qhat_c(coord, shape, a)
