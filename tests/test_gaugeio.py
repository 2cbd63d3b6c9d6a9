"""Gauge-file readers: a literal loop-by-loop restatement of the reference's
Fortran readers (src/gaugeIO/openqcdfileio_standalone.f90:29-95,
src/gaugeIO/ILDG_bin.f90:14-105) read the same bytes as the vectorised
readers, and write -> read round trips are exact."""
import numpy as np
import pytest

from flue_gb300 import gaugeIO, generate


def _fortran_openqcd_read(path):
    """Direct restatement of ReadGaugeField_OpenQCD's loops (without
    FixSU3Matrix, which the comparison applies to both sides)."""
    raw = open(path, "rb").read()
    nt, nx, ny, nz = np.frombuffer(raw[:16], "<i4")
    pos = 24
    U = np.zeros((nt, nx, ny, nz, 4, 3, 3), np.complex128)
    modc = lambda a, b: (a - 1) % b + 1  # noqa: E731
    for it in range(1, nt + 1):
        for ix in range(1, nx + 1):
            for iy in range(1, ny + 1):
                for iz in range(1, nz + 1):
                    if (ix + iy + iz + it - 4) % 2 == 0:
                        continue
                    for idd in range(1, 5):
                        mu = modc(idd - 1, 4)
                        dmu = [0, 0, 0, 0]
                        dmu[mu - 1] = 1
                        jx = modc(ix - dmu[0], nx)
                        jy = modc(iy - dmu[1], ny)
                        jz = modc(iz - dmu[2], nz)
                        jt = modc(it - dmu[3], nt)
                        for (a, b, c, d) in ((it, ix, iy, iz), (jt, jx, jy, jz)):
                            m = np.frombuffer(raw[pos:pos + 144], "<c16")
                            pos += 144
                            utmp = m.reshape(3, 3, order="F")  # Fortran read of UTmp(3,3)
                            U[a - 1, b - 1, c - 1, d - 1, mu - 1] = utmp.T  # TRANSPOSE (:237-238)
    return np.roll(U, 1, axis=4)  # CSHIFT(U, -1, dim=5) (:93)


def _fortran_ildg_read(path, nx, ny, nz, nt):
    raw = np.fromfile(path, ">c16")
    per = 9 * 4 * nx * ny * nz
    U = np.zeros((nt, nx, ny, nz, 4, 3, 3), np.complex128)
    nu_of = {1: 2, 2: 3, 3: 4, 4: 1}
    for it in range(nt):
        rec = raw[it * per:(it + 1) * per].reshape((3, 3, 4, nx, ny, nz), order="F")  # URead(:,:,:,:,:,:,it)
        for ix in range(nx):
            for iy in range(ny):
                for iz in range(nz):
                    for mu in range(1, 5):
                        U[it, ix, iy, iz, nu_of[mu] - 1] = rec[:, :, mu - 1, ix, iy, iz].T
    return U


@pytest.fixture(scope="module")
def field():
    return generate.random_field((4, 2, 4, 2), 0.6, 77)


def test_openqcd_needs_even_extents(tmp_path):
    with pytest.raises(ValueError):
        gaugeIO.write_openqcd(tmp_path / "x", generate.random_field((4, 2, 3, 2), 0.6, 1))


def test_openqcd_reader_matches_fortran_loops(field, tmp_path):
    p = tmp_path / "cfg.openqcd"
    gaugeIO.write_openqcd(p, field, plaq=0.75)
    U, hdr = gaugeIO.read_openqcd(p, return_header=True)
    assert hdr["dims"] == field.shape[:4] and hdr["plaq"] == 0.75
    ref = generate._reunitarise_np(_fortran_openqcd_read(p))
    assert np.abs(U - ref).max() < 1e-15
    assert np.abs(U - field).max() < 1e-14


def test_ildg_reader_matches_fortran_loops(field, tmp_path):
    p = tmp_path / "cfg.ildg"
    gaugeIO.write_ildg_be(p, field)
    nt, nx, ny, nz = field.shape[:4]
    U = gaugeIO.read_ildg_be(p, nx, ny, nz, nt)
    ref = generate._reunitarise_np(_fortran_ildg_read(p, nx, ny, nz, nt))
    assert np.abs(U - ref).max() < 1e-15
    assert np.abs(U - field).max() < 1e-14


def test_cola_transformation_round_trip(tmp_path):
    G = generate.random_gauge_transform((3, 2, 2, 4), 5)
    p = tmp_path / "fix.gag"
    gaugeIO.write_gauge_transformation_cola(p, G)
    G2 = gaugeIO.read_gauge_transformation_cola(p, 2, 2, 4, 3)
    assert np.abs(G2 - G).max() < 1e-14


def test_reader_rejects_truncated_file(field, tmp_path):
    p = tmp_path / "cfg.ildg"
    gaugeIO.write_ildg_be(p, field)
    with open(p, "r+b") as fh:
        fh.truncate(100)
    with pytest.raises(ValueError):
        gaugeIO.read_ildg_be(p, 2, 4, 2, 4)


@pytest.mark.gpu
def test_device_ingest_matches_host(field, tmp_path):
    p = tmp_path / "cfg.openqcd"
    gaugeIO.write_openqcd(p, field)
    host = gaugeIO.read_openqcd(p)
    dev = gaugeIO.read_openqcd(p, device="cuda")
    assert np.abs(dev.to_numpy() - host).max() < 1e-15
    q = tmp_path / "cfg.ildg"
    gaugeIO.write_ildg_be(q, field)
    nt, nx, ny, nz = field.shape[:4]
    d2 = gaugeIO.read_ildg_be(q, nx, ny, nz, nt, device="cuda", prec="r12")
    assert np.abs(d2.to_numpy() - host).max() < 1e-6
