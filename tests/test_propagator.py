"""Gluon propagator oracle and analysis helpers (CPU).

The oracle (oracle/propagator.py) is pinned to closed forms: a cold field
has D = 0; a constant abelian field has D only at q = 0; a single Fourier
mode of an abelian field has D only at +-k, with the amplitude the
normalisation fixes; a global gauge rotation leaves D unchanged; the FFT
agrees with the direct Fourier sum.  The gluonAna helpers are checked
against literal loop restatements of src/gluonAna/gpManip.f90."""
import numpy as np
import pytest

from flue_gb300 import generate, gluonAna
from oracle import propagator as P


def _abelian(theta):
    """U_mu(x) = diag(e^{i theta}, e^{-i theta}, 1) for theta[t,x,y,z,mu]."""
    U = np.zeros(theta.shape + (3, 3), np.complex128)
    U[..., 0, 0] = np.exp(1j * theta)
    U[..., 1, 1] = np.exp(-1j * theta)
    U[..., 2, 2] = 1.0
    return U


def test_cold_field_zero():
    U = generate.cold_field((4, 3, 2, 5))
    assert np.abs(P.gluon_propagator(U)).max() == 0.0


@pytest.mark.parametrize("xi,mu_start", [(1.0, 0), (1.7, 0), (1.7, 1)])
def test_constant_abelian(xi, mu_start):
    dims = (4, 3, 4, 2)
    th = np.array([0.3, -0.2, 0.5, 0.7])
    U = _abelian(np.broadcast_to(th, dims + (4,)).copy())
    D = P.gluon_propagator(U, xi, mu_start)
    V = np.prod(dims)
    w = np.array([xi * xi, 1, 1, 1])
    w[:mu_start] = 0
    # A^3_mu = 2 sin(theta_mu) everywhere: A^3_mu(0) = 2 V sin(theta_mu)
    expect0 = np.sum(w * (2 * V * np.sin(th)) ** 2) / (8 * 4 * V)
    assert abs(D[0, 0, 0, 0] - expect0) < 1e-12 * expect0
    D[0, 0, 0, 0] = 0
    assert np.abs(D).max() < 1e-12 * expect0


@pytest.mark.parametrize("nu,xi", [(0, 1.3), (2, 1.0)])
def test_single_mode(nu, xi):
    dims = (6, 4, 5, 4)
    n = np.array([1, 2, 0, 1])
    grids = np.meshgrid(*[np.arange(k) for k in dims], indexing="ij")
    phase = sum(2 * np.pi * n[d] * grids[d] / dims[d] for d in range(4))
    s = 0.4
    theta = np.zeros(dims + (4,))
    theta[..., nu] = np.arcsin(s * np.cos(phase))  # A^3_nu = 2 s cos(k.x)
    D = P.gluon_propagator(_abelian(theta), xi)
    V = np.prod(dims)
    w = xi * xi if nu == 0 else 1.0
    expect = w * (s * V) ** 2 / (8 * 3 * V)
    kp = tuple(n % np.array(dims))
    km = tuple((-n) % np.array(dims))
    assert abs(D[kp] - expect) < 1e-12 * expect and abs(D[km] - expect) < 1e-12 * expect
    D[kp] = D[km] = 0
    assert np.abs(D).max() < 1e-12 * expect


def test_fft_matches_direct_sum_and_global_gauge_invariance():
    U = generate.random_field((3, 4, 2, 3), 0.6, 4)
    D = P.gluon_propagator(U, 1.2, 0)
    assert np.abs(D - P.gluon_propagator_dft(U, 1.2, 0)).max() < 1e-13 * np.abs(D).max()
    g = generate.random_gauge_transform((1, 1, 1, 1), 9)[0, 0, 0, 0]
    Ug = np.einsum("ij,...jk,lk->...il", g, U, np.conj(g))
    assert np.abs(P.gluon_propagator(Ug, 1.2, 0) - D).max() < 1e-12 * np.abs(D).max()


# --- gluonAna against literal restatements of gpManip.f90 -------------------
def _q_average_loops(NQ, q, D, q_slices):
    dout, qout = np.zeros(NQ + 1), np.zeros(NQ + 1)
    maxq = max(q)
    dq = maxq / float(q_slices)
    q_pos, qcount = 0.0, 1
    while True:
        sel = [i for i in range(NQ) if q[i] > q_pos and q[i] < q_pos + dq]
        if sel:
            acc = 0.0
            for i in sel:
                acc = acc + float(q[i])
            qout[qcount - 1] = acc / len(sel)
            dout[qcount - 1] = D[0]
            qcount += 1
        q_pos = q_pos + dq
        if q_pos + dq >= maxq:
            break
    return dout, qout, qcount


def _cone_cut_loops(NQ, radius, Q, D, D4, angle, xi, ircut, irradius):
    keep = []
    for qq in range(NQ):
        qh = list(Q[qq])
        q_norm = np.sqrt(sum(v * v for v in qh))
        qh[0] = qh[0] * xi
        if all(v == qh[0] for v in qh):
            r = theta = 0.0
        else:
            c = sum(0.5 * v for v in qh) / q_norm
            theta = np.arccos(c) if abs(c) <= 1 else np.nan
            r = q_norm * np.sin(theta)
        keep.append(r <= irradius if q_norm <= ircut else (r <= irradius and theta < angle))
    idx = [i for i in range(NQ) if keep[i]]
    return Q[idx], D[idx], D4[idx], len(idx)


def test_q_average_matches_loops():
    rng = np.random.default_rng(3)
    q = rng.uniform(0, 5, 200)
    D = rng.uniform(0, 1, 200)
    d1, q1, c1 = gluonAna.q_average(200, q, D, 17, stat="first")
    d2, q2, c2 = _q_average_loops(200, q, D, 17)
    assert c1 == c2 and np.array_equal(q1, q2) and np.array_equal(d1, d2)
    dm, qm, cm = gluonAna.q_average(200, q, D, 17, stat="mean")
    assert cm == c1 and np.array_equal(qm, q1)
    k = 0
    dq = q.max() / 17
    # the first kept bin's mean of D
    m = (q > 0) & (q < dq)
    assert abs(dm[k] - D[m].mean()) < 1e-15


def test_cone_cut_matches_loops():
    qh = gluonAna.momenta((8, 4, 4, 4)).reshape(-1, 4)
    n = len(qh)
    rng = np.random.default_rng(5)
    D, D4 = rng.uniform(size=n), rng.uniform(size=n)
    for angle, xi, ircut, irr in ((np.pi / 2, 1.0, 0.0, 1.0), (0.4, 2.0, 1.0, 0.5), (1.0, 1.0, 10.0, 0.3)):
        qo, do, d4o, c = gluonAna.cone_cut(n, 1, qh, D, D4, 8, 4, angle, xi, ircut, irr)
        q2, d2, d42, c2 = _cone_cut_loops(n, 1, qh, D, D4, angle, xi, ircut, irr)
        assert c == c2 and c > 0
        assert np.array_equal(qo[:c], q2) and np.array_equal(do[:c], d2) and np.array_equal(d4o[:c], d42)
        assert not qo[c:].any()


def test_get_qhat_and_momenta():
    assert np.allclose(gluonAna.get_qhat([1, 2, 0, 3], [8, 4, 4, 6]), 2 * np.pi * np.array([1 / 8, 0.5, 0, 0.5]))
    m = gluonAna.momenta((4, 3, 2, 5))
    assert m.shape == (4, 3, 2, 5, 4)
    assert np.isclose(m[3, 0, 0, 0, 0], -2 * np.pi / 4) and np.isclose(m[2, 0, 0, 0, 0], np.pi)
