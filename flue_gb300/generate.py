"""Seeded synthetic SU(3) gauge fields (no real ensembles are needed or used).

* ``random_field(dims, eps, seed)``: every link is exp(i eps H) with
  H = sum_a c_a lambda_a / 2, c_a ~ N(0,1) drawn from numpy's
  ``PCG64(seed)`` in (t, x, y, z, mu, a) order, lambda_a the Gell-Mann
  matrices; the result is reunitarised with FixSU3Matrix's Gram-Schmidt
  (which fixes det = 1).
* ``haar_field(dims, seed)``: Haar-random SU(3) links from the QR
  decomposition of complex Gaussian matrices with the phases of R's diagonal
  moved into Q, then det fixed to 1 and reunitarised.
* ``cold_field(dims)``: U = 1.

Fields come back as Fortran-ordered numpy complex128 arrays
``data[t,x,y,z,mu,a,b]`` (the reference's memory layout), or, with
``device="cuda"``, as :class:`~flue_gb300.field.GaugeField` objects whose
exponentials are formed on the GPU (torch ``matrix_exp``) -- the random
numbers are always drawn on the host, so both paths use the same c_a.
"""
from __future__ import annotations

import numpy as np

GELL_MANN = np.zeros((8, 3, 3), dtype=np.complex128)
GELL_MANN[0][0, 1] = GELL_MANN[0][1, 0] = 1
GELL_MANN[1][0, 1] = -1j
GELL_MANN[1][1, 0] = 1j
GELL_MANN[2][0, 0] = 1
GELL_MANN[2][1, 1] = -1
GELL_MANN[3][0, 2] = GELL_MANN[3][2, 0] = 1
GELL_MANN[4][0, 2] = -1j
GELL_MANN[4][2, 0] = 1j
GELL_MANN[5][1, 2] = GELL_MANN[5][2, 1] = 1
GELL_MANN[6][1, 2] = -1j
GELL_MANN[6][2, 1] = 1j
GELL_MANN[7][0, 0] = GELL_MANN[7][1, 1] = 1 / np.sqrt(3)
GELL_MANN[7][2, 2] = -2 / np.sqrt(3)


def _shape(dims):
    nt, nx, ny, nz = (int(d) for d in dims)
    return (nt, nx, ny, nz, 4)


def _reunitarise_np(u: np.ndarray) -> np.ndarray:
    """FixSU3Matrix (src/gaugeIO/ILDG_bin.f90:138-151) vectorised over (...,3,3)."""
    v1 = u[..., 0, :].copy()
    v1 /= np.sqrt(np.sum(v1.real ** 2 + v1.imag ** 2, axis=-1))[..., None]
    v2 = u[..., 1, :].copy()
    d = np.sum(np.conj(v1) * v2, axis=-1)
    v2 -= v1 * d[..., None]
    v2 /= np.sqrt(np.sum(v2.real ** 2 + v2.imag ** 2, axis=-1))[..., None]
    v3 = np.conj(np.cross(v1, v2))
    v3 /= np.sqrt(np.sum(v3.real ** 2 + v3.imag ** 2, axis=-1))[..., None]
    out = np.empty_like(u)
    out[..., 0, :] = v1
    out[..., 1, :] = v2
    out[..., 2, :] = v3
    return out


def _to_fortran_field(links: np.ndarray) -> np.ndarray:
    """(NT,NX,NY,NZ,4,3,3) C-ordered -> same indices, Fortran memory order."""
    return np.asfortranarray(links)


def gell_mann_coeffs(dims, seed: int) -> np.ndarray:
    rng = np.random.Generator(np.random.PCG64(seed))
    return rng.standard_normal(_shape(dims) + (8,))


def hermitian_from_coeffs(c: np.ndarray) -> np.ndarray:
    return np.einsum("...a,aij->...ij", c, GELL_MANN) * 0.5


def random_field(dims, eps: float, seed: int, device=None):
    c = gell_mann_coeffs(dims, seed)
    if device is not None:
        import torch

        from .field import GaugeField

        h = torch.as_tensor(hermitian_from_coeffs(c)).to(device)
        u = torch.linalg.matrix_exp(1j * eps * h)
        return GaugeField.from_array(u, prec="c128", reunitarise=True)
    h = hermitian_from_coeffs(c)
    w, v = np.linalg.eigh(h)
    u = np.einsum("...ij,...j,...kj->...ik", v, np.exp(1j * eps * w), np.conj(v))
    return _to_fortran_field(_reunitarise_np(u))


def random_field_philox(dims, eps: float, seed: int, device="cuda", prec="c128"):
    """Like :func:`random_field` but with the Gell-Mann coefficients drawn on
    the GPU from torch's Philox generator seeded with ``seed`` (for large
    ensembles, where host generation would dominate).  Deterministic for a
    given seed and torch build; not the same numbers as the PCG64 path."""
    import torch

    from .field import GaugeField

    g = torch.Generator(device=device)
    g.manual_seed(int(seed))
    c = torch.randn(_shape(dims) + (8,), generator=g, device=device, dtype=torch.float64)
    lam = torch.as_tensor(GELL_MANN, device=device)
    h = torch.einsum("...a,aij->...ij", c.to(torch.complex128), lam) * 0.5
    del c
    u = torch.linalg.matrix_exp(1j * eps * h)
    del h
    return GaugeField.from_array(u, prec=prec, reunitarise=True)


def haar_field(dims, seed: int, device=None):
    rng = np.random.Generator(np.random.PCG64(seed))
    z = (rng.standard_normal(_shape(dims) + (3, 3)) + 1j * rng.standard_normal(_shape(dims) + (3, 3))) / np.sqrt(2)
    if device is not None:
        import torch

        from .field import GaugeField

        zt = torch.as_tensor(z).to(device)
        q, r = torch.linalg.qr(zt)
        d = torch.diagonal(r, dim1=-2, dim2=-1)
        q = q * (d / d.abs()).unsqueeze(-2)
        det = torch.linalg.det(q)
        q = q / (det ** (1.0 / 3.0)).unsqueeze(-1).unsqueeze(-1)
        return GaugeField.from_array(q, prec="c128", reunitarise=True)
    q, r = np.linalg.qr(z)
    d = np.diagonal(r, axis1=-2, axis2=-1)
    q = q * (d / np.abs(d))[..., None, :]
    det = np.linalg.det(q)
    q = q / (det ** (1.0 / 3.0))[..., None, None]
    return _to_fortran_field(_reunitarise_np(q))


def cold_field(dims, device=None):
    u = np.zeros(_shape(dims) + (3, 3), dtype=np.complex128)
    u[..., 0, 0] = u[..., 1, 1] = u[..., 2, 2] = 1
    if device is not None:
        from .field import GaugeField

        return GaugeField.from_array(np.asfortranarray(u))
    return _to_fortran_field(u)


def random_gauge_transform(dims, seed: int, eps: float = 1.0) -> np.ndarray:
    """Random SU(3) matrices G(x), shape (NT,NX,NY,NZ,3,3), Fortran order."""
    nt, nx, ny, nz = dims
    rng = np.random.Generator(np.random.PCG64(seed))
    c = rng.standard_normal((nt, nx, ny, nz, 8))
    h = hermitian_from_coeffs(c)
    w, v = np.linalg.eigh(h)
    g = np.einsum("...ij,...j,...kj->...ik", v, np.exp(1j * eps * w), np.conj(v))
    return np.asfortranarray(_reunitarise_np(g))


def random_su3_algebra(shape, seed: int) -> np.ndarray:
    """Random traceless anti-Hermitian matrices X = sum_a x_a T^a,
    T^a = i lambda_a / 2, x_a ~ N(0,1); shape (...,3,3)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    x = rng.standard_normal(tuple(shape) + (8,))
    return 1j * np.einsum("...a,aij->...ij", x, GELL_MANN) * 0.5
