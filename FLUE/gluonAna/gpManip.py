"""python/FLUE/gluonAna/gpManip.py over the GB300 build's flue_c.

The reference's wrappers pass NQ (and, for q_average, the output arrays)
positionally; f2py infers NQ from the arrays and returns the intent(out)
values, which is what these functions return."""
from FLUE.compiled import flue_c as fc


def q_average(NQ, q, D, q_slices, DOUT=None, QOUT=None, Qcount=None):
    """(DOUT, QOUT, Qcount); the output arguments of the reference's call
    are accepted and ignored (f2py returns intent(out) values)."""
    return fc.q_average_c(q, D, q_slices, nq=NQ)


def cone_cut(NQ, radius, Q, D, D4, NT, NS, angleIN, xiIN, IRCutIN, IRRadiusIN):
    """(QOUT, Dout, D4out, qcount)"""
    return fc.cone_cut_c(radius, Q, D, D4, NT, NS, angleIN, xiIN, IRCutIN, IRRadiusIN, nq=NQ)
