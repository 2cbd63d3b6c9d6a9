"""A reference user's calls through ``import FLUE`` against the oracle: the
f2py-style ``FLUE.compiled.flue_c`` (host numpy field in, numpy out) and
``FLUE.gluonCalc`` (numpy field, or a field already on the GPU), FP64 to
1e-12 as the other parity tests."""
import numpy as np
import pytest

import FLUE
import oracle
from FLUE.compiled import flue_c
from flue_gb300 import generate
from flue_gb300.field import GaugeField

pytestmark = pytest.mark.gpu


def rel(a, b):
    return abs(a - b) / max(abs(b), 1e-300)


@pytest.fixture(scope="module")
def U():
    return generate.random_field((8, 4, 6, 4), 0.4, 77)


def test_flue_c_reference_calls(U):
    s, n, t = flue_c.plaquette(U, 1, 4, 4)
    so, no = oracle.plaquette(U, 1, 4, 4)
    assert n == no and rel(s, so) < 1e-12 and t >= 0
    assert flue_c.genplaquette(U, 2, 4, 4)[:2] == flue_c.plaquette(U, 2, 4, 4)[:2]
    s, n, _ = flue_c.polyakov(U)
    so, no = oracle.polyakov(U)
    assert n == no and abs(s - so) < 1e-12 * n
    assert rel(flue_c.magnetic(U), oracle.magnetic(U)) < 1e-12
    q = flue_c.loop5munucoord(U, 3, 2)
    assert q.shape == U.shape[:4] + (3, 3) and q.flags.f_contiguous
    assert np.abs(q - oracle.loop5munucoord(U, 3, 2)).max() < 1e-12
    c = flue_c.cloverloopmunucoord(U, 1, 4)
    assert np.abs(c - oracle.cloverloopmunucoord(U, 1, 4)).max() < 1e-12
    path = [2, 3, -2, 4, -3, -4, 1]
    assert np.abs(flue_c.genericpath(U, [2, 1, 3, 4], path) - oracle.genericpath(U, [2, 1, 3, 4], path)).max() < 1e-13
    assert abs(flue_c.wmunu(U, 2, 3, 2, 3) - oracle.wmunu(U, 2, 3, 2, 3)) < 1e-12
    assert abs(flue_c.wmunutau(U, 3, 1, 4, 1, 2) - oracle.wmunutau(U, 3, 1, 4, 1, 2)) < 1e-12
    g = generate.random_gauge_transform(U.shape[:4], 5)
    assert np.abs(flue_c.uzerobar(U, g) - oracle.uzerobar(U, g)).max() < 1e-12
    a, b = U[0, 0, 0, 0, 1], U[3, 1, 2, 0, 2]
    assert np.abs(flue_c.multiplymatmat_c(a, b) - oracle.multiplymatmat(a, b)).max() < 1e-14
    m = np.asfortranarray(U[1, 1, 1, 1, 3] * (1 + 1e-3))
    want = oracle.fixsu3matrix(m)
    flue_c.fixsu3matrix(m)
    assert np.abs(m - want).max() < 1e-14
    # a C-ordered or complex64 input is converted, as f2py converts intent(in) arrays
    assert rel(flue_c.magnetic(np.ascontiguousarray(U)), oracle.magnetic(U)) < 1e-12


def test_gluoncalc_numpy_and_device_fields(U):
    bo = oracle.magnetic(U)
    assert rel(FLUE.gluonCalc.magnetic(U), bo) < 1e-12
    f = GaugeField.from_array(U)
    assert rel(FLUE.gluonCalc.magnetic(f), bo) < 1e-12
    s, n, _ = FLUE.gluonCalc.plaquette(f, 1, 1, 4)
    so, no = oracle.plaquette(U, 1, 1, 4)
    assert n == no and rel(s, so) < 1e-12
    q = FLUE.gluonCalc.loop5munucoord(f, 2, 4)
    assert np.abs(q.cpu().numpy() - oracle.loop5munucoord(U, 2, 4)).max() < 1e-12
    a, b = U[0, 1, 0, 0, 1], U[2, 1, 2, 0, 3]
    assert np.abs(FLUE.gluonCalc.multiplymatmat(a, b) - a @ b).max() < 1e-14
    b2, grad = FLUE.gluonCalc.magnetic_force(U)
    go = oracle.loop5_energy_force(U, oracle.B2_PLANES)
    assert rel(b2, bo) < 1e-12 and np.abs(grad - go).max() < 1e-11 * np.abs(go).max()
    b32, g32 = flue_c.magnetic_force(U, prec="r12")
    assert rel(b32, bo) < 1e-6
    assert np.linalg.norm(g32 - go) < 1e-6 * np.linalg.norm(go)


def test_gluon_propagator_entries():
    from oracle import propagator as P

    U = generate.random_field((6, 4, 4, 4), 0.3, 12)
    D = FLUE.gluonCalc.scalarGluonProp(U, 1.0)
    ref = P.gluon_propagator(U, 1.0, 0)
    assert D.shape == (6, 4, 4, 4) and np.abs(D - ref).max() < 1e-12 * max(1.0, np.abs(ref).max())
    Dq = FLUE.gluonCalc.calc_mom_space_scalarD(U, 1, 1.0)
    ref1 = P.gluon_propagator(U, 1.0, 1)[:4, :3, :3, :3]
    assert Dq.shape == (4, 3, 3, 3) and Dq.dtype == np.complex128
    assert np.abs(Dq.real - ref1).max() < 1e-12 * max(1.0, np.abs(ref1).max()) and not Dq.imag.any()
