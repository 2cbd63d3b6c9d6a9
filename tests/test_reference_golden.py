"""The oracle against golden vectors of the reference's own routines.

`tests/golden/reference_fortran.json` holds the outputs of the reference's
`src/SU3MatrixOps.f90` and `src/wloops.F90`, run as written through the
Fortran-subset translator (`tests/golden/fortran_subset.py`, generated by
`tests/golden/make_reference_golden.py`): plaquettes (`plaquette`,
`genPlaquette`), `polyakov`, `genericPath`, `wmunu`, `wmunutau`,
`cloverLoopMuNuCoord`, `Loop5MuNuCoord`, `magnetic`, the 3x3 helpers and
`FixSU3Matrix` (`src/gaugeIO/ILDG_bin.f90`), on a
random field, a Haar field and the 8^3 x 16 field of the plain-method
benchmark case.  Every value of the C oracle must agree to FP64 rounding.
The analysis helpers of `src/jack.f90` and `src/gluonAna/*.f90`, run the same
way on seeded inputs, pin `flue_gb300.jack` and `flue_gb300.gluonAna`; the
gauge-file readers of `src/gaugeIO/*.f90`, run on ILDG, openQCD and cola
files written by `flue_gb300.gaugeIO`, pin its readers.
"""
import json
import os

import numpy as np
import pytest

import oracle
from tests.golden.make_reference_golden import checksum, field, field_summary

GOLD_PATH = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "reference_fortran.json")
GOLD = json.load(open(GOLD_PATH))
TOL = 1e-12
CASES = sorted(GOLD["fields"])


def cx(pair, shape=None):
    a = np.asarray(pair[0]) + 1j * np.asarray(pair[1])
    return a.reshape(shape, order="F") if shape else a


def close(got, want, tol=TOL):
    got, want = np.asarray(got), np.asarray(want)
    scale = max(1.0, float(np.max(np.abs(want))))
    return float(np.max(np.abs(got - want))) <= tol * scale


def check_summary(F, want, tol=TOL):
    got = field_summary(np.asarray(F))
    assert close(got["checksum"], want["checksum"], tol), (got["checksum"], want["checksum"])
    for k, m in want["sites"].items():
        assert close(cx(got["sites"][k]), cx(m), tol), k


@pytest.fixture(scope="module", params=CASES)
def case(request):
    g = GOLD["fields"][request.param]
    U = field(g["recipe"])
    # the seeded field is the one the golden vectors were made from
    assert close(checksum(U), g["checksum"], 1e-13)
    return request.param, U, g


def test_algebra_helpers():
    a = GOLD["algebra"]
    m = [cx(p, (3, 3)) for p in a["matrices"]]
    assert close(oracle.multiplymatmat(m[0], m[1]), cx(a["multiplymatmat"], (3, 3)))
    assert close(oracle.multiplymatdagmatdag(m[2], m[3]), cx(a["multiplymatdagmatdag"], (3, 3)))
    # RealTraceMultMatMat = Re Tr(left right)
    assert close(np.real(np.trace(m[0] @ m[3])), a["realtracemultmatmat"])
    # FixSU3Matrix (src/gaugeIO/ILDG_bin.f90)
    for mi, mo in zip(a["fixsu3matrix"]["in"], a["fixsu3matrix"]["out"]):
        assert close(oracle.fixsu3matrix(cx(mi, (3, 3))), cx(mo, (3, 3)), 1e-13)


def test_plaquettes(case):
    name, U, g = case
    for rng, w in g["plaquette"].items():
        r = tuple(int(v) for v in rng.split(","))
        s, n = oracle.plaquette(U, *r)
        assert n == w["n"] and close(s, w["sum"]), (name, rng)
        s, n = oracle.genplaquette(U, *r)
        assert n == w["gen_n"] and close(s, w["gen_sum"]), (name, rng)


def test_polyakov(case):
    name, U, g = case
    if "polyakov" not in g:
        pytest.skip("the reference defines the Polyakov loop for NT >= 3 only")
    s, n = oracle.polyakov(U)
    assert n == g["polyakov"]["n"] and close(s, g["polyakov"]["sum"]), name


def test_generic_paths(case):
    name, U, g = case
    for p in g["genericpath"]:
        assert close(oracle.genericpath(U, p["coord"], p["path"]), cx(p["matrix"], (3, 3))), (name, p["path"])


def test_wilson_loops(case):
    name, U, g = case
    for w in g["wmunu"]:
        assert close(oracle.wmunu(U, *w["args"]), w["value"]), (name, w["args"])
    for w in g["wmunutau"]:
        assert close(oracle.wmunutau(U, *w["args"]), w["value"]), (name, w["args"])


def test_field_strength(case):
    name, U, g = case
    for c in g.get("clover", []):
        check_summary(oracle.cloverloopmunucoord(U, *c["plane"]), c)
    for c in g.get("loop5", []):
        check_summary(oracle.loop5munucoord(U, *c["plane"]), c)


def test_magnetic(case):
    name, U, g = case
    assert close(oracle.magnetic(U), g["magnetic"]), name


# --- analysis helpers (src/jack.f90, src/gluonAna/momentum.f90, gpManip.f90) ---


def test_jackknife():
    from flue_gb300 import jack

    a = GOLD["analysis"]
    d = np.asarray(a["data"])
    assert close(jack.complement(d), a["complement0"])
    assert close(jack.complement(d, ("all",)), a["complement1"])
    c2 = a["complement2"]
    assert close(jack.complement(d, (c2["icon"] - 1,)), c2["value"])
    c3 = a["complement3"]
    assert close(jack.complement(d, (c3["icon"] - 1, c3["jcon"] - 1)), c3["value"])
    err, bias = jack.jackknife_wp(a["jackknife"]["c"])
    assert close(err, a["jackknife"]["err"]) and close(bias, a["jackknife"]["bias"])


def test_momenta_and_qhat():
    from flue_gb300 import gluonAna

    for g in GOLD["analysis"]["get_qhat"]:
        assert close(gluonAna.get_qhat(g["coord"], g["shape"], g["a"]), g["qhat"])


def test_q_average():
    from flue_gb300 import gluonAna

    qa = GOLD["analysis"]["q_average"]
    q, D = np.asarray(qa["q"]), np.asarray(qa["D"])
    for run in qa["runs"]:
        # the reference's DOUT is D(1) in every bin ("first")
        dout, qout, qcount = gluonAna.q_average(q.size, q, D, run["q_slices"], stat="first")
        assert qcount == run["qcount"]
        assert close(qout, run["qout"]) and close(dout, run["dout"])


def test_cone_cut():
    from flue_gb300 import gluonAna

    cc = GOLD["analysis"]["cone_cut"]
    dims = tuple(cc["lattice"])
    Q = gluonAna.momenta(dims).transpose(3, 2, 1, 0, 4).reshape(-1, 4)  # rows with time fastest
    D, D4 = np.asarray(cc["D"]), np.asarray(cc["D4"])
    names = ("angleIN", "xiIN", "IRCutIN", "IRRadiusIN")
    for run in cc["runs"]:
        kw = {k: v for k, v in zip(names, run["angle_xi_ircut_irradius"]) if v is not None}
        qout, dout, d4out, qcount = gluonAna.cone_cut(Q.shape[0], run["radius"], Q, D, D4, dims[0], dims[1], **kw)
        assert qcount == run["qcount"]
        n = qcount
        assert close(qout[:n].ravel(order="F"), run["qout"])
        assert close(dout[:n], run["dout"]) and close(d4out[:n], run["d4out"])


# --- gauge-file readers (src/gaugeIO/ILDG_bin.f90, openqcdfileio_standalone.f90) ---


def test_gauge_file_readers(tmp_path):
    from flue_gb300 import gaugeIO
    from tests.golden.make_reference_golden import write_reader_files

    r = GOLD["readers"]
    nt, nx, ny, nz = r["recipe"]["dims"]
    paths = write_reader_files(r["recipe"], str(tmp_path))
    got = {"ildg": np.asarray(gaugeIO.read_ildg_be(paths["ildg"], nx, ny, nz, nt)),
           "openqcd": np.asarray(gaugeIO.read_openqcd(paths["openqcd"]))}
    for key, U in got.items():
        want = r[key]
        assert close(checksum(U), want["checksum"]), key
        flat = U.reshape((-1, 3, 3), order="F")
        for k, m in want["links"].items():
            assert close(flat[int(k)], cx(m, (3, 3))), (key, k)
    G = np.asarray(gaugeIO.read_gauge_transformation_cola(paths["cola"], nx, ny, nz, nt))
    check_summary(G, r["cola"])
