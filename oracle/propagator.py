"""CPU oracle of the scalar gluon propagator (test infrastructure only; the
same import rules as the rest of ``oracle``).

The reference's propagator code (``src/gluonCalc/gluonProp.f90``,
``colourDecomp`` at ``src/SU3MatrixOps.f90:107-122``) is unfinished and
cannot serve as an oracle (out-of-bounds reads at q = 0, Fourier sums that
ignore their loop indices, a colour decomposition that keeps only real
parts).  This module restates the definition it works towards, that of
hep-lat/9803105 (cited at ``gluonProp.f90:38``), independently of the GPU
formulation: explicit Gell-Mann matrices, ``numpy.fft.fftn`` over the four
lattice axes (and a direct O(V^2) Fourier sum for tiny lattices):

    A_mu(x)   = [U_mu(x) - U_mu(x)^+] / (2i) - Tr/3
    A^a_mu(q) = sum_x exp(-i q.x) Tr(A_mu(x) lambda^a),   q_mu = 2 pi n_mu / N_mu
    D(q)      = 2 / ((Nc^2 - 1) n(q) V) sum_{mu >= mu_start} w_mu Tr[A_mu(q) A_mu(-q)]

with w_t = xi^2, w_i = 1, n(0) = 4 and n(q != 0) = 3
(``gluonProp.f90:186-190, 208-236``).  Parity against the reference's own
outputs is unpinned; the oracle is pinned to closed forms (cold field,
constant and single-mode abelian fields) in ``tests/test_oracle.py``.

Fields are ``complex128`` arrays ``U[t,x,y,z,mu,a,b]``; D is indexed
``D[nt,nx,ny,nz]`` with n_mu = 0..N_mu-1.
"""
from __future__ import annotations

import numpy as np


def gell_mann() -> np.ndarray:
    """The eight Gell-Mann matrices lambda^1..lambda^8, shape (8, 3, 3)."""
    lam = np.zeros((8, 3, 3), dtype=np.complex128)
    lam[0][0, 1] = lam[0][1, 0] = 1
    lam[1][0, 1], lam[1][1, 0] = -1j, 1j
    lam[2][0, 0], lam[2][1, 1] = 1, -1
    lam[3][0, 2] = lam[3][2, 0] = 1
    lam[4][0, 2], lam[4][2, 0] = -1j, 1j
    lam[5][1, 2] = lam[5][2, 1] = 1
    lam[6][1, 2], lam[6][2, 1] = -1j, 1j
    lam[7] = np.diag([1, 1, -2]) / np.sqrt(3)
    return lam


def colour_fields(U: np.ndarray) -> np.ndarray:
    """A^a_mu(x) = Tr(A_mu(x) lambda^a), real, shape (NT,NX,NY,NZ,4,8)."""
    U = np.asarray(U, dtype=np.complex128)
    A = (U - np.conj(np.swapaxes(U, -1, -2))) / 2j
    tr = np.trace(A, axis1=-2, axis2=-1)
    A = A - tr[..., None, None] * np.eye(3) / 3
    comp = np.einsum("...ij,aji->...a", A, gell_mann())
    return comp.real


def _normalise(S: np.ndarray) -> np.ndarray:
    V = S.size
    n = np.full(S.shape, 3.0)
    n[0, 0, 0, 0] = 4.0
    return S / (8.0 * n * V)


def _weights(xi: float, mu_start: int) -> np.ndarray:
    w = np.array([xi * xi, 1.0, 1.0, 1.0])
    w[:mu_start] = 0.0
    return w


def gluon_propagator(U: np.ndarray, xi: float = 1.0, mu_start: int = 0) -> np.ndarray:
    """D(q) on every momentum by numpy's FFT (sign exp(-i q.x))."""
    a = colour_fields(U)
    F = np.fft.fftn(a, axes=(0, 1, 2, 3))
    S = np.einsum("...ma,m->...", np.abs(F) ** 2, _weights(xi, mu_start))
    return _normalise(S)


def gluon_propagator_dft(U: np.ndarray, xi: float = 1.0, mu_start: int = 0) -> np.ndarray:
    """The same by the direct Fourier sum (O(V^2): tiny lattices only)."""
    a = colour_fields(U)
    dims = a.shape[:4]
    grids = np.meshgrid(*[np.arange(n) for n in dims], indexing="ij")
    x = np.stack([g.reshape(-1) for g in grids], axis=1)  # (V, 4) coordinates
    q = 2 * np.pi * x / np.array(dims)  # (V, 4) momenta, same enumeration
    phase = np.exp(-1j * q @ x.T)  # (Vq, Vx)
    F = phase @ a.reshape(len(x), -1)  # (Vq, 32)
    S = (np.abs(F.reshape(len(x), 4, 8)) ** 2).sum(axis=2) @ _weights(xi, mu_start)
    return _normalise(S.reshape(dims))
