"""Pinning of the CPU oracle (no GPU): analytic known answers, an
independent numpy restatement, symmetry properties and the committed
regression fixtures."""
import json
import math
import os

import numpy as np
import pytest

import oracle
from flue_gb300 import generate
from tests import np_flue
from tests.golden.make_golden import abelian_field, KAT_CASES

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def _rel(a, b):
    return abs(a - b) / max(1e-300, abs(b))


# ---------------------------------------------------------------------------
# analytic known answers
# ---------------------------------------------------------------------------
@pytest.mark.parametrize("idx", range(len(KAT_CASES)))
def test_abelian_known_answers(idx):
    kat = json.load(open(os.path.join(GOLD, "abelian_kat.json")))[idx]
    U = abelian_field(kat["case"])
    ex = kat["expected"]
    assert _rel(oracle.plaquette(U, 1, 4, 4)[0], ex["plaq_all"]) < 1e-13
    assert _rel(oracle.plaquette(U, 2, 4, 4)[0], ex["plaq_spatial"]) < 1e-13
    assert _rel(oracle.plaquette(U, 1, 1, 4)[0], ex["plaq_temporal"]) < 1e-13
    assert _rel(oracle.genplaquette(U, 1, 4, 4)[0], ex["plaq_all"]) < 1e-13
    assert abs(oracle.polyakov(U)[0] - ex["polyakov"]) < 1e-11 * np.prod(kat["case"]["dims"][1:])
    for key, val in ex["wmunu_23"].items():
        r, t = (int(v) for v in key.split(","))
        assert abs(oracle.wmunu(U, 2, 3, r, t) - val) < 1e-12
    fc = oracle.cloverloopmunucoord(U, 2, 3)
    f5 = oracle.loop5munucoord(U, 2, 3)
    for a in range(3):
        assert np.allclose(fc[..., a, a], 1j * ex["clover_diag_im"][a], atol=1e-13)
        assert np.allclose(f5[..., a, a], 1j * ex["loop5_diag_im"][a], atol=1e-13)
    off = ~np.eye(3, dtype=bool)
    assert np.abs(f5[..., off]).max() < 1e-14
    assert abs(oracle.magnetic(U) - ex["magnetic"]) < 1e-12


def test_cold_field():
    U = generate.cold_field((4, 3, 3, 5))
    V = 4 * 3 * 3 * 5
    assert oracle.plaquette(U, 1, 4, 4) == (18.0 * V, 6 * V)
    assert oracle.plaquette(U, 2, 4, 4) == (9.0 * V, 3 * V)
    assert oracle.polyakov(U) == (3.0 * 45, 45)
    assert oracle.wmunu(U, 1, 3, 2, 2) == 3.0
    assert np.all(oracle.loop5munucoord(U, 3, 2) == 0)
    assert oracle.magnetic(U) == 0.0


def test_five_loop_coefficients_normalised():
    # k1 + 4 k2 + 9 k5 + 2 k3 + 3 k4 = 1 (continuum normalisation)
    k = np_flue
    assert abs(k.K1 + 4 * k.K2 + 9 * k.K5 + 2 * k.K3 + 3 * k.K4 - 1.0) < 1e-15


# ---------------------------------------------------------------------------
# independent numpy restatement
# ---------------------------------------------------------------------------
@pytest.fixture(scope="module")
def rnd():
    return generate.random_field((4, 3, 4, 5), 0.4, 7)


def test_numpy_restatement_paths(rnd):
    for path in ([1, 2, -1, -2], [2, 2, 3, -2, -4, -3, 1], [-3, 4, 4, 1, -4]):
        a = oracle.genericpath_all(rnd, path)
        b = np_flue.genericpath_all(rnd, path)
        assert np.abs(a - b).max() < 1e-13
    g = oracle.genericpath(rnd, [2, 3, 1, 4], [1, -2, 3])
    b = np_flue.genericpath_all(rnd, [1, -2, 3])[1, 2, 0, 3]
    assert np.abs(g - b).max() < 1e-14


def test_numpy_restatement_observables(rnd):
    for r in ((1, 4, 4), (2, 4, 4), (1, 1, 4), (2, 3, 4)):
        assert _rel(oracle.plaquette(rnd, *r)[0], np_flue.plaquette(rnd, *r)[0]) < 1e-13
    re, im, n = np_flue.polyakov(rnd)
    assert abs(oracle.polyakov(rnd)[0] - re) < 1e-12
    assert abs(oracle.wmunu(rnd, 2, 4, 2, 3) - np_flue.wmunu(rnd, 2, 4, 2, 3)) < 1e-13
    for mu, nu in ((3, 2), (1, 4)):
        assert np.abs(oracle.loop5munucoord(rnd, mu, nu) - np_flue.loop5munucoord(rnd, mu, nu)).max() < 1e-13
        assert np.abs(oracle.cloverloopmunucoord(rnd, mu, nu) - np_flue.cloverloopmunucoord(rnd, mu, nu)).max() < 1e-13
    assert _rel(oracle.magnetic(rnd), np_flue.magnetic(rnd)) < 1e-12
    assert _rel(oracle.magnetic(rnd, parallel=True), np_flue.magnetic(rnd)) < 1e-12


def test_genericpath_is_transposed_product():
    U = generate.random_field((3, 3, 3, 3), 0.8, 3)
    g = oracle.genericpath(U, [1, 1, 1, 1], [2, 3])
    prod = U[0, 0, 0, 0, 1] @ U[0, 1, 0, 0, 2]
    assert np.abs(g - prod.T).max() < 1e-15


def test_multiplymatmat():
    rng = np.random.default_rng(1)
    a = rng.standard_normal((3, 3)) + 1j * rng.standard_normal((3, 3))
    b = rng.standard_normal((3, 3)) + 1j * rng.standard_normal((3, 3))
    assert np.abs(oracle.multiplymatmat(a, b) - a @ b).max() < 1e-14
    # the reference's code forms L^+ R^+ (its comment says (L R)^+)
    assert np.abs(oracle.multiplymatdagmatdag(a, b) - np.conj(a).T @ np.conj(b).T).max() < 1e-14


def test_fixsu3_matches_numpy():
    rng = np.random.default_rng(2)
    m = rng.standard_normal((3, 3)) + 1j * rng.standard_normal((3, 3))
    f = oracle.fixsu3matrix(m)
    assert np.abs(f @ np.conj(f).T - np.eye(3)).max() < 1e-14
    assert abs(np.linalg.det(f) - 1) < 1e-14
    assert np.abs(f - generate._reunitarise_np(m)).max() < 1e-14


# ---------------------------------------------------------------------------
# symmetries
# ---------------------------------------------------------------------------
def _gauge(U, G):
    """U'_mu(x) = G(x) U_mu(x) G(x+mu)^+"""
    out = np.empty_like(U)
    for mu in range(4):
        off = [0, 0, 0, 0]
        off[mu] = 1
        out[..., mu, :, :] = G @ U[..., mu, :, :] @ np_flue.dag(np_flue.shift(G, off))
    return np.asfortranarray(out)


def test_gauge_invariance_and_covariance(rnd):
    G = generate.random_gauge_transform(rnd.shape[:4], 5)
    Ug = _gauge(rnd, G)
    assert _rel(oracle.plaquette(Ug, 1, 4, 4)[0], oracle.plaquette(rnd, 1, 4, 4)[0]) < 1e-13
    assert _rel(oracle.polyakov(Ug)[0], oracle.polyakov(rnd)[0]) < 1e-12
    assert _rel(oracle.wmunu(Ug, 1, 3, 2, 2), oracle.wmunu(rnd, 1, 3, 2, 2)) < 1e-12
    assert _rel(oracle.magnetic(Ug), oracle.magnetic(rnd)) < 1e-12
    # F transforms as G F G^+; genericPath transposes: F^T -> conj(G) F^T G^T
    f = oracle.loop5munucoord(rnd, 2, 4)
    fg = oracle.loop5munucoord(Ug, 2, 4)
    pred = np.conj(G) @ f @ np.swapaxes(G, -1, -2)
    assert np.abs(fg - pred).max() < 1e-12


def test_translation_invariance(rnd):
    Ur = np.asfortranarray(np.roll(rnd, shift=(1, 2, 0, 3), axis=(0, 1, 2, 3)))
    assert _rel(oracle.plaquette(Ur, 1, 4, 4)[0], oracle.plaquette(rnd, 1, 4, 4)[0]) < 1e-13
    assert _rel(oracle.magnetic(Ur), oracle.magnetic(rnd)) < 1e-12


def test_haar_field_statistics():
    """Haar-random SU(3) links: every plaquette and Polyakov loop is itself
    Haar distributed, so E Re Tr = 0 and Var Re Tr = 1/2; the lattice averages
    vanish within 5 standard errors, and the links are special unitary."""
    U = generate.haar_field((6, 6, 6, 6), 11)
    eye = np.eye(3)
    assert np.abs(U @ np.conj(np.swapaxes(U, -1, -2)) - eye).max() < 1e-13
    assert np.abs(np.linalg.det(U) - 1).max() < 1e-13
    for rng in ((1, 4, 4), (2, 4, 4), (1, 1, 4)):
        s, n = oracle.plaquette(U, *rng)
        assert abs(s / n) < 5 * math.sqrt(0.5 / n), rng
    s, n = oracle.polyakov(U)
    assert abs(s / n) < 5 * math.sqrt(0.5 / n)


def test_centre_symmetry(rnd):
    z = np.exp(2j * math.pi / 3)
    Uc = rnd.copy(order="F")
    Uc[2, ..., 0, :, :] *= z
    re, im, _ = np_flue.polyakov(rnd)
    rot = (complex(re, im) * z).real
    assert abs(oracle.polyakov(Uc)[0] - rot) < 1e-12
    assert _rel(oracle.plaquette(Uc, 2, 4, 4)[0], oracle.plaquette(rnd, 2, 4, 4)[0]) < 1e-13


def test_polyakov_rejects_short_time_extent():
    with pytest.raises(ValueError):
        oracle.polyakov(generate.cold_field((2, 2, 2, 2)))


# ---------------------------------------------------------------------------
# gradients: finite differences and the analytic staple force
# ---------------------------------------------------------------------------
def _perturb(U, X, h):
    E = np_flue.expm_su3(h * X)
    return np.asfortranarray(E @ U)


def _lie_pair(G, X):
    # D_X O = sum -2 Re Tr(X G)
    return float(-2.0 * np.einsum("...ij,...ji->...", X, G).real.sum())


def test_plaquette_staple_force_fd():
    U = generate.random_field((3, 3, 4, 3), 0.5, 21)
    G = oracle.plaquette_staple_force(U)
    X = generate.random_su3_algebra(U.shape[:5], 3)
    h = 1e-4
    fd = (oracle.plaquette(_perturb(U, X, h), 1, 4, 4)[0] - oracle.plaquette(_perturb(U, X, -h), 1, 4, 4)[0]) / (2 * h)
    assert _rel(_lie_pair(G, X), fd) < 1e-7
    # gradient is traceless anti-Hermitian
    assert np.abs(G + np_flue.dag(G)).max() < 1e-14
    assert np.abs(np.trace(G, axis1=-2, axis2=-1)).max() < 1e-14


@pytest.mark.parametrize("planes", [oracle.B2_PLANES, oracle.ALL_PLANES])
def test_loop5_energy_force_fd(planes):
    U = generate.random_field((3, 4, 3, 3), 0.5, 22)
    G = oracle.loop5_energy_force(U, planes)
    X = generate.random_su3_algebra(U.shape[:5], 4)
    h = 1e-4
    e = lambda V: oracle.loop5_energy(V, planes)  # noqa: E731
    fd = (e(_perturb(U, X, h)) - e(_perturb(U, X, -h))) / (2 * h)
    assert _rel(_lie_pair(G, X), fd) < 1e-6
    if planes == oracle.B2_PLANES:
        assert np.abs(G[..., 0, :, :]).max() == 0.0
        assert _rel(oracle.loop5_energy(U, planes), oracle.magnetic(U)) < 1e-13


# ---------------------------------------------------------------------------
# committed regression fixtures
# ---------------------------------------------------------------------------
def test_regression_fixtures():
    recs = json.load(open(os.path.join(GOLD, "oracle_regression.json")))
    for rec in recs:
        U = generate.random_field(rec["dims"], rec["eps"], rec["seed"])
        assert _rel(oracle.plaquette(U, 1, 4, 4)[0], rec["plaq_all"]) < 1e-13
        assert _rel(oracle.polyakov(U)[0], rec["polyakov"]) < 1e-12
        assert _rel(oracle.magnetic(U), rec["magnetic"]) < 1e-12
        assert _rel(oracle.wmunu(U, 2, 3, 2, 3), rec["wmunu_23_2_3"]) < 1e-12
        assert _rel(oracle.wmunutau(U, 2, 1, 4, 1, 2), rec["wmunutau_2_14_1_2"]) < 1e-12
        g = oracle.genericpath(U, [2, 1, 3, 1], [1, 2, -1, 3, -2, -3, 4])
        ref = np.array([complex(*v) for v in rec["genericpath"]]).reshape(3, 3)
        assert np.abs(g - ref).max() < 1e-13


def test_uzerobar_definitions():
    U = generate.random_field((4, 3, 3, 3), 0.3, 31)
    u = oracle.uzerobar(U)
    p_all = oracle.plaquette(U, 1, 4, 4)
    assert abs(u[0] - (p_all[0] / p_all[1] / 3) ** 0.25) < 1e-14
    assert np.all(np.isnan(u[3:]))
    # identity gauge transformation -> mean link of U itself
    G = np.zeros(U.shape[:4] + (3, 3), dtype=np.complex128)
    G[..., 0, 0] = G[..., 1, 1] = G[..., 2, 2] = 1
    u2 = oracle.uzerobar(U, np.asfortranarray(G))
    ml = np.trace(U, axis1=-2, axis2=-1).real.mean() / 3
    assert abs(u2[3] - ml) < 1e-14
    # a cold field in a random gauge has mean link 1 after gauge fixing back
    C = generate.cold_field(U.shape[:4])
    Gr = generate.random_gauge_transform(U.shape[:4], 9)
    Cg = _gauge(C, Gr)
    u3 = oracle.uzerobar(Cg, np.asfortranarray(np_flue.dag(Gr)))
    assert np.allclose(u3, 1.0, atol=1e-13)
