"""The ``FLUE`` drop-in package on the CPU: it imports like the reference's
package (``import FLUE``, ``FLUE.compiled.flue_c``, ``FLUE.gluonCalc``,
``FLUE.gluonAna``), keeps f2py's calling conventions, and its host-only
analysis routines agree with their definitions.  The GPU routines are
checked against the oracle in tests/test_gpu_flue_dropin.py."""
import numpy as np
import pytest

import FLUE
from FLUE.compiled import flue_c
from flue_gb300 import gluonAna


def test_package_layout_matches_the_reference():
    # python/FLUE/__init__.py:1-4, gluonCalc/__init__.py:1-4, gluonAna/__init__.py:1-5
    assert set(FLUE.__all__) == {"gluonAna", "gluonCalc"}
    for name in ("multiplymatmat", "calc_mom_space_scalarD", "scalarGluonProp"):
        assert callable(getattr(FLUE.gluonCalc, name))
    for name in ("q_average", "get_qhat", "cone_cut"):
        assert callable(getattr(FLUE.gluonAna, name))
    # the routines of c_wrapper/FLUE_c.f90 under their f2py (lower-case) names
    for name in ("scalargluonprop_c", "calc_mom_space_scalard_c", "multiplymatmat_c", "q_average_c", "get_qhat_c",
                 "cone_cut_c"):
        assert callable(getattr(flue_c, name))
    # the wloops routines of the hot path
    for name in ("plaquette", "genplaquette", "polyakov", "genericpath", "wmunu", "wmunutau", "cloverloopmunucoord",
                 "loop5munucoord", "magnetic", "uzerobar", "fixsu3matrix"):
        assert callable(getattr(flue_c, name)) and getattr(flue_c, name + "_c") is getattr(flue_c, name)
        assert callable(getattr(FLUE.gluonCalc, name))


def test_get_qhat_definition():
    # src/gluonAna/momentum.f90:8-24: 2 pi coord / (a shape)
    q = FLUE.gluonAna.get_qhat([1, 2, 3, 4], [8, 8, 8, 16])
    assert np.allclose(q, 2 * np.pi * np.array([1, 2, 3, 4]) / np.array([8, 8, 8, 16]), rtol=0, atol=1e-15)
    q2 = flue_c.get_qhat_c([1, 0, 0, 0], [4, 4, 4, 4], 0.5)
    assert abs(q2[0] - 2 * np.pi / 0.5 / 4) < 1e-15
    with pytest.raises(ValueError):
        flue_c.get_qhat_c([1, 2, 3], [4, 4, 4, 4])


def test_q_average_and_cone_cut_follow_the_f2py_outputs():
    rng = np.random.default_rng(4)
    q = rng.uniform(0.1, 3.0, 40)
    D = rng.uniform(0.0, 5.0, 40)
    dout, qout, qc = FLUE.gluonAna.q_average(40, q, D, 7)
    d2, q2, c2 = gluonAna.q_average(40, q, D, 7, stat="first")
    assert qc == c2 and np.array_equal(qout, q2) and np.array_equal(dout, d2)
    # the reference's DOUT is D(1) for every kept bin (src/gluonAna/gpManip.f90:38)
    assert np.all(dout[: qc - 1] == D[0])
    Q = rng.uniform(-2, 2, (30, 4))
    D4 = rng.uniform(0, 1, 30)
    qo, do, d4o, n = FLUE.gluonAna.cone_cut(30, 1, Q, D[:30], D4, 8, 4, np.pi / 3, 1.0, 0.5, 1.0)
    ref = gluonAna.cone_cut(30, 1, Q, D[:30], D4, 8, 4, np.pi / 3, 1.0, 0.5, 1.0)
    assert n == ref[3] and np.array_equal(qo, ref[0]) and np.array_equal(do, ref[1]) and np.array_equal(d4o, ref[2])


def test_shape_and_dtype_errors_before_any_device_work():
    bad = np.zeros((4, 4, 4, 4, 4, 3, 2), dtype=np.complex128)
    for fn, args in ((flue_c.plaquette, (1, 4, 4)), (flue_c.polyakov, ()), (flue_c.magnetic, ()),
                     (flue_c.loop5munucoord, (3, 2)), (flue_c.wmunu, (2, 3, 1, 1))):
        with pytest.raises(ValueError):
            fn(bad, *args)
    good = np.zeros((4, 4, 4, 4, 4, 3, 3), dtype=np.complex128, order="F")
    with pytest.raises(ValueError):
        flue_c.plaquette(good, 1, 4, 4, nt=5)  # an explicit extent must match the array
    with pytest.raises(ValueError):
        flue_c.multiplymatmat_c(np.eye(2), np.eye(3))
    with pytest.raises(ValueError):
        flue_c.fixsu3matrix(np.ascontiguousarray(np.eye(3, dtype=np.complex128)))  # C order: not inout-able
    with pytest.raises(ValueError):
        flue_c.fixsu3matrix(np.eye(3))  # float64, not complex128: intent(inout) refuses a copy
