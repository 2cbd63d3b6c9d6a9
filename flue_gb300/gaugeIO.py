"""Gauge-field file formats of the reference's readers, and device ingest.

Readers follow src/gaugeIO/openqcdfileio_standalone.f90 (openQCD,
little-endian stream) and src/gaugeIO/ILDG_bin.f90 (ILDG binary, big-endian,
one record per time slice; cola gauge transformation), vectorised with
numpy; the result is the reference's ``U(NT,NX,NY,NZ,4,3,3)`` with
direction 1 = t, reunitarised link by link with FixSU3Matrix.  With
``device=...`` the byte-order fix-up happens on the host and the re-layout
and FixSU3Matrix run in one GPU kernel (``flue_pack_field``).

Writers produce the same formats (used for round-trip tests and to hand
fields to the reference's tools).
"""
from __future__ import annotations

import numpy as np

from .generate import _reunitarise_np

__all__ = ["read_openqcd", "write_openqcd", "read_ildg_be", "write_ildg_be", "read_gauge_transformation_cola",
           "write_gauge_transformation_cola"]


def _finish(U: np.ndarray, device, prec, reunitarise=True):
    """U: [t,x,y,z,mu,a,b] complex128 host array, not yet reunitarised."""
    if device is None:
        if reunitarise:
            U = _reunitarise_np(U)
        return np.asfortranarray(U)
    from .field import GaugeField

    return GaugeField.from_array(U, prec=prec or "c128", reunitarise=reunitarise, device=device)


# ---------------------------------------------------------------------------
# openQCD (src/gaugeIO/openqcdfileio_standalone.f90:29-95)
# ---------------------------------------------------------------------------
def _odd_sites(nt, nx, ny, nz):
    if any(n % 2 for n in (nt, nx, ny, nz)):
        # odd sites + backward links cover every link only on an even lattice
        raise ValueError(f"openQCD format needs even lattice extents, got {(nt, nx, ny, nz)}")
    t, x, y, z = np.meshgrid(np.arange(nt), np.arange(nx), np.arange(ny), np.arange(nz), indexing="ij")
    odd = ((t + x + y + z) % 2) == 1  # the file skips sites with (ix+iy+iz+it-4) even (:55)
    return t[odd], x[odd], y[odd], z[odd]  # in t, x, y, z order with z fastest (:51-54)


def read_openqcd(path, device=None, prec=None, return_header=False):
    """openQCD configuration: header (NT,NX,NY,NZ: int32, plaq: float64),
    then for every odd site and direction t,x,y,z the forward link and the
    link arriving from the backward neighbour, each a row-major 3x3 complex
    matrix, little-endian."""
    with open(path, "rb") as fh:
        hdr = np.frombuffer(fh.read(16), dtype="<i4")
        plaq = float(np.frombuffer(fh.read(8), dtype="<f8")[0])
        nt, nx, ny, nz = (int(v) for v in hdr)
        raw = np.frombuffer(fh.read(), dtype="<c16")
    t, x, y, z = _odd_sites(nt, nx, ny, nz)
    n = t.size
    if raw.size != n * 4 * 2 * 9:
        raise ValueError(f"openQCD file {path}: expected {n * 72} matrices' elements, found {raw.size}")
    m = raw.reshape(n, 4, 2, 3, 3).astype(np.complex128)
    U = np.zeros((nt, nx, ny, nz, 4, 3, 3), dtype=np.complex128)
    ext = (nt, nx, ny, nz)
    for d in range(4):
        U[t, x, y, z, d] = m[:, d, 0]
        back = [t.copy(), x.copy(), y.copy(), z.copy()]
        back[d] = (back[d] - 1) % ext[d]
        U[back[0], back[1], back[2], back[3], d] = m[:, d, 1]
    out = _finish(U, device, prec)
    return (out, {"dims": ext, "plaq": plaq}) if return_header else out


def write_openqcd(path, U, plaq: float = 0.0):
    """Write U[t,x,y,z,mu,a,b] in the openQCD layout read by read_openqcd."""
    U = np.asarray(U)
    nt, nx, ny, nz = U.shape[:4]
    t, x, y, z = _odd_sites(nt, nx, ny, nz)
    ext = (nt, nx, ny, nz)
    m = np.empty((t.size, 4, 2, 3, 3), dtype="<c16")
    for d in range(4):
        m[:, d, 0] = U[t, x, y, z, d]
        back = [t.copy(), x.copy(), y.copy(), z.copy()]
        back[d] = (back[d] - 1) % ext[d]
        m[:, d, 1] = U[back[0], back[1], back[2], back[3], d]
    with open(path, "wb") as fh:
        fh.write(np.asarray([nt, nx, ny, nz], dtype="<i4").tobytes())
        fh.write(np.asarray([plaq], dtype="<f8").tobytes())
        fh.write(m.tobytes())


# ---------------------------------------------------------------------------
# ILDG binary, big-endian (src/gaugeIO/ILDG_bin.f90:14-63)
# ---------------------------------------------------------------------------
_ILDG_TO_FLUE = (3, 0, 1, 2)  # FLUE direction d (t,x,y,z) <- ILDG index (x,y,z,t) (:45-54)


def read_ildg_be(path, nx, ny, nz, nt, device=None, prec=None):
    """ILDG binary data, big-endian: time slices in order, within a slice
    x fastest, then y, z; per site the four directions x,y,z,t, each a
    row-major 3x3 complex matrix."""
    raw = np.fromfile(path, dtype=">c16")
    if raw.size != nt * nz * ny * nx * 4 * 9:
        raise ValueError(f"ILDG file {path}: size does not match {nx}x{ny}x{nz}x{nt}")
    r = raw.reshape(nt, nz, ny, nx, 4, 3, 3)
    U = np.empty((nt, nx, ny, nz, 4, 3, 3), dtype=np.complex128)
    for d in range(4):
        U[..., d, :, :] = r[..., _ILDG_TO_FLUE[d], :, :].transpose(0, 3, 2, 1, 4, 5)
    return _finish(U, device, prec)


def write_ildg_be(path, U):
    U = np.asarray(U)
    nt, nx, ny, nz = U.shape[:4]
    r = np.empty((nt, nz, ny, nx, 4, 3, 3), dtype=">c16")
    for d in range(4):
        r[..., _ILDG_TO_FLUE[d], :, :] = U[..., d, :, :].transpose(0, 3, 2, 1, 4, 5)
    r.tofile(path)


# ---------------------------------------------------------------------------
# cola gauge transformation (src/gaugeIO/ILDG_bin.f90:65-105): Fortran
# sequential unformatted, big-endian, 4-byte record markers; records
# Re(G^T[:,:,:,:,:,1]), Im(...), Re(G^T[...,2]), Im(...) with G^T indexed
# (x,y,z,t,colour) x fastest -- the first two rows of G.
# ---------------------------------------------------------------------------
def _read_records(path, endian=">"):
    recs = []
    with open(path, "rb") as fh:
        data = fh.read()
    pos = 0
    while pos < len(data):
        n = int(np.frombuffer(data[pos:pos + 4], dtype=endian + "u4")[0])
        recs.append(data[pos + 4:pos + 4 + n])
        pos += 8 + n
    return recs


def read_gauge_transformation_cola(path, nx, ny, nz, nt):
    """G(NT,NX,NY,NZ,3,3): rows 1 and 2 from the file, row 2 orthogonalised
    against row 1, row 3 = conj(row1 x row2) (no normalisation, as in the
    reference, :93-102)."""
    recs = _read_records(path)
    if len(recs) != 4:
        raise ValueError(f"cola file {path}: expected 4 records, found {len(recs)}")
    shape = (3, nt, nz, ny, nx)  # Fortran (x,y,z,t,c) -> C order reversed
    re1, im1, re2, im2 = (np.frombuffer(r, dtype=">f8").reshape(shape) for r in recs)
    v1 = (re1 + 1j * im1).transpose(1, 4, 3, 2, 0)  # (t,x,y,z,c)
    v2 = (re2 + 1j * im2).transpose(1, 4, 3, 2, 0)
    d = np.sum(np.conj(v1) * v2, axis=-1)
    v2 = v2 - v1 * d[..., None]
    v3 = np.conj(np.cross(v1, v2))
    G = np.stack([v1, v2, v3], axis=-2)
    return np.asfortranarray(G.astype(np.complex128))


def write_gauge_transformation_cola(path, G):
    G = np.asarray(G)
    with open(path, "wb") as fh:
        for row in (0, 1):
            v = G[..., row, :].transpose(4, 0, 3, 2, 1)  # (c,t,z,y,x)
            for part in (v.real, v.imag):
                b = np.ascontiguousarray(part, dtype=">f8").tobytes()
                m = np.asarray([len(b)], dtype=">u4").tobytes()
                fh.write(m + b + m)
