"""Host-side analysis helpers of the gluon propagator, the counterpart of the
reference's ``FLUE.gluonAna`` (python/FLUE/gluonAna/__init__.py:1-5;
src/gluonAna/momentum.f90, src/gluonAna/gpManip.f90).  They act on small
arrays of momenta and propagator values after the GPU measurement, so they
are numpy code.  Arguments and results follow the f2py conventions of the
reference's wrappers (c_wrapper/FLUE_c.f90:38-77): intent(out) values are
returned, output arrays keep the Fortran sizes and are zero beyond the count.
"""
from __future__ import annotations

import numpy as np


def get_qhat(coord, shape, a: float = 1.0) -> np.ndarray:
    """q^_mu = (2 pi / a) coord_mu / shape_mu (src/gluonAna/momentum.f90:8-24)."""
    return (2.0 * np.pi / a) * np.asarray(coord, dtype=np.float64) / np.asarray(shape, dtype=np.float64)


def momenta(dims, a: float = 1.0) -> np.ndarray:
    """q^ of every momentum index of a lattice (NT,NX,NY,NZ), shape
    (NT,NX,NY,NZ,4), with n_mu > N_mu/2 taken as the negative momenta
    n_mu - N_mu (the Fourier index convention of the propagator)."""
    axes = []
    for n in dims:
        k = np.arange(n)
        axes.append(np.where(k > n // 2, k - n, k))
    grid = np.stack(np.meshgrid(*axes, indexing="ij"), axis=-1)
    return get_qhat(grid, np.asarray(dims), a)


def q_average(NQ, q, D, q_slices, stat: str = "median"):
    """Q_Average(NQ, q, D, q_slices) -> (DOUT, QOUT, Qcount)
    (src/gluonAna/gpManip.f90:10-49): bins (q_pos, q_pos + dq) of width
    dq = max(q)/q_slices, open at both ends, stepping until q_pos + dq >= max(q)
    (the last full bin is not visited, as in the reference); QOUT holds the
    mean q of every non-empty bin.  The reference's DOUT is a placeholder
    (D(1) for every bin, :38, with the median and mean it meant commented
    out): stat = "median" (default) or "mean" of D in the bin, or "first"
    for the reference's values.  Qcount is the reference's counter: bins
    kept + 1.  DOUT, QOUT have NQ + 1 entries."""
    q = np.asarray(q, dtype=np.float64)[:NQ]
    D = np.asarray(D, dtype=np.float64)[:NQ]
    dout = np.zeros(NQ + 1)
    qout = np.zeros(NQ + 1)
    maxq = q.max()
    dq = maxq / float(q_slices)
    q_pos = 0.0
    qcount = 1
    while True:
        mask = (q > q_pos) & (q < q_pos + dq)
        if mask.any():
            # plain sequential sum, as Fortran's SUM (not pairwise, not compensated)
            qout[qcount - 1] = float(np.cumsum(q[mask])[-1]) / int(mask.sum())
            if stat == "first":
                dout[qcount - 1] = D[0]
            elif stat == "mean":
                dout[qcount - 1] = D[mask].mean()
            elif stat == "median":
                dout[qcount - 1] = np.median(D[mask])
            else:
                raise ValueError("stat must be 'median', 'mean' or 'first'")
            qcount += 1
        q_pos = q_pos + dq
        if q_pos + dq >= maxq:
            break
    return dout, qout, qcount


def cone_cut(NQ, radius, Q, D, D4, NT, NS, angleIN=np.pi / 2.0, xiIN=1.0, IRCutIN=0.0, IRRadiusIN=None):
    """cone_cut(...) -> (QOUT, DOUT, D4OUT, qcount) (src/gluonAna/gpManip.f90:51-163):
    keep the momenta within distance IRRadius (default: radius) of the
    diagonal (1,1,1,1)/2 and, above |q| = IRCut, within angle of it; the
    time component is scaled by xi first (:120), the norm is taken before
    the scaling (:112), on-diagonal points have r = theta = 0 (:124-127).
    NT, NS are accepted as in the reference and not used there either."""
    Q = np.asarray(Q, dtype=np.float64)[:NQ]
    D = np.asarray(D, dtype=np.float64)[:NQ]
    D4 = np.asarray(D4, dtype=np.float64)[:NQ]
    ir_radius = float(radius) if IRRadiusIN is None else float(IRRadiusIN)
    bcd = np.full(4, 0.5)
    q_norm = np.sqrt(np.sum(Q ** 2, axis=1))
    qh = Q.copy()
    qh[:, 0] = qh[:, 0] * xiIN
    diag = np.all(qh == qh[:, :1], axis=1)
    with np.errstate(invalid="ignore", divide="ignore"):
        theta = np.where(diag, 0.0, np.arccos((qh @ bcd) / q_norm))
        r = np.where(diag, 0.0, q_norm * np.sin(theta))
    keep = np.where(q_norm <= IRCutIN, r <= ir_radius, (r <= ir_radius) & (theta < angleIN))
    qcount = int(keep.sum())
    qout = np.zeros((NQ, 4))
    dout = np.zeros(NQ)
    d4out = np.zeros(NQ)
    qout[:qcount] = Q[keep]
    dout[:qcount] = D[keep]
    d4out[:qcount] = D4[keep]
    return qout, dout, d4out, qcount
