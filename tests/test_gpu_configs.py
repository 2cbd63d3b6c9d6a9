"""GPU parity on the benchmark's stated configurations, against the oracle.

* The plain-method configuration: an 8^3 x 16 periodic lattice, links
  exp(i 0.3 H) from PCG64 seed 1 (``generate.random_field``), every
  observable of the path in FP64 to 1e-12 and in FP32 (complex64 and
  reconstruct-12) to the FP32 bounds written below.
* The FP32 accuracy bound of the headline (B^2 and its su(3) gradient within
  1e-6 relative of the FP64 oracle) on a 16^3 x 32 lattice, eps 0.3, for both
  FP32 field formats; the gradient is compared as a relative L2 norm over
  the whole field.
* The full-size 32^3 x 64 lattice on a Haar-random (strong-coupling) field:
  plaquettes, Polyakov loop, B^2 and u0 against the oracle in FP64, and the
  FP32 B^2 bound.  The other full-size fields (eps 0.1 and 0.5) and the
  remaining observables at that size are covered by the validation run
  ``python tests/validation_report.py config1``.
"""
import numpy as np
import pytest
import torch

import oracle
from flue_gb300 import forces, generate, gluonCalc as G
from flue_gb300.field import GaugeField

pytestmark = pytest.mark.gpu

CONFIG0 = ((16, 8, 8, 8), 0.3, 1)  # (NT, NX, NY, NZ), eps, PCG64 seed
FP32_BOUND = 1e-6  # relative error of FP32 B^2 and of its gradient (L2) against FP64
PATHS = ([1, 2, -1, -2], [2, 2, 3, -4, -2, 1, 1, -3], [-1, -1, 4, 3, 3, 3, -2], [3, 3, 3, 2, -3, -3, -3, -2])
ALL_PLANES = ((1, 2), (1, 3), (1, 4), (2, 3), (2, 4), (3, 4))


def rel(a, b):
    return abs(a - b) / max(abs(b), 1e-300)


def _np(x):
    return x.detach().cpu().numpy() if isinstance(x, torch.Tensor) else np.asarray(x)


@pytest.fixture(scope="module")
def U0():
    dims, eps, seed = CONFIG0
    return generate.random_field(dims, eps, seed)


@pytest.fixture(scope="module")
def grad0(U0):
    return oracle.loop5_energy_force(U0, oracle.B2_PLANES)


def test_config0_fp64_every_observable(U0, grad0):
    U = U0
    f = GaugeField.from_array(U)
    for r in ((1, 4, 4), (2, 4, 4), (1, 1, 4)):
        s, n, _ = G.plaquette(f, *r)
        so, no = oracle.plaquette(U, *r)
        assert n == no and rel(s, so) < 1e-12, r
        assert G.genplaquette(f, *r)[:2] == (s, n)
    s, n, _ = G.polyakov(f)
    so, no = oracle.polyakov(U)
    assert n == no and abs(s - so) < 1e-12 * n
    for path in PATHS:
        assert np.abs(_np(G.genericpath_all(f, path)) - oracle.genericpath_all(U, path)).max() < 1e-12
        for cb in ([1, 1, 1, 1], [16, 8, 3, 5]):
            assert np.abs(_np(G.genericpath(f, cb, path)) - oracle.genericpath(U, cb, path)).max() < 1e-12
    tab = _np(G.wmunu_table(f, 2, 3, 8, 8))
    for r in range(8):
        for t in range(8):
            assert abs(tab[r, t] - oracle.wmunu(U, 2, 3, r + 1, t + 1)) < 1e-12, (r, t)
    for args in ((1, 4, 3, 5), (4, 1, 2, 8)):
        assert abs(G.wmunu(f, *args) - oracle.wmunu(U, *args)) < 1e-12
    for tau in (1, 16):
        assert abs(G.wmunutau(f, tau, 2, 4, 2, 3) - oracle.wmunutau(U, tau, 2, 4, 2, 3)) < 1e-12
    for mu, nu in ALL_PLANES:
        assert np.abs(_np(G.cloverloopmunucoord(f, mu, nu)) - oracle.cloverloopmunucoord(U, mu, nu)).max() < 1e-12
        assert np.abs(_np(G.loop5munucoord(f, mu, nu)) - oracle.loop5munucoord(U, mu, nu)).max() < 1e-12
    b = G.magnetic(f)
    bo = oracle.magnetic(U)
    assert rel(b, bo) < 1e-12
    g = generate.random_gauge_transform(U.shape[:4], 8)
    assert np.abs(G.uzerobar(f, g) - oracle.uzerobar(U, g)).max() < 1e-12
    b2, grad = forces.magnetic_force(f)
    go = grad0
    assert rel(b2, bo) < 1e-12
    assert np.abs(_np(grad) - go).max() < 1e-11 * np.abs(go).max()
    _, gp = forces.plaquette_force(f)
    assert np.abs(_np(gp) - oracle.plaquette_staple_force(U)).max() < 1e-12


@pytest.mark.parametrize("prec", ["c64", "r12"])
def test_config0_fp32_every_observable(U0, grad0, prec):
    """FP32 link products with FP64 sums: bounds relative to the observable
    (sums) or to the largest element (matrix fields)."""
    U = U0
    f = GaugeField.from_array(U, prec=prec)
    for r in ((1, 4, 4), (2, 4, 4), (1, 1, 4)):
        s, n, _ = G.plaquette(f, *r)
        so, no = oracle.plaquette(U, *r)
        assert n == no and rel(s, so) < 1e-6, r
    s, n, _ = G.polyakov(f)
    so, no = oracle.polyakov(U)
    assert abs(s - so) < 1e-6 * n
    for path in PATHS:
        assert np.abs(_np(G.genericpath_all(f, path)) - oracle.genericpath_all(U, path)).max() < 2e-6
    tab = _np(G.wmunu_table(f, 2, 3, 8, 8))
    for r, t in ((0, 0), (3, 5), (7, 7)):
        assert abs(tab[r, t] - oracle.wmunu(U, 2, 3, r + 1, t + 1)) < 2e-6, (r, t)
    for mu, nu in ALL_PLANES:
        c = oracle.cloverloopmunucoord(U, mu, nu)
        assert np.abs(_np(G.cloverloopmunucoord(f, mu, nu)) - c).max() < 2e-6 * np.abs(c).max()
        q = oracle.loop5munucoord(U, mu, nu)
        assert np.abs(_np(G.loop5munucoord(f, mu, nu)) - q).max() < 2e-6 * np.abs(q).max()
    bo = oracle.magnetic(U)
    assert rel(G.magnetic(f), bo) < FP32_BOUND
    b2, grad = forces.magnetic_force(f)
    go = grad0
    g = _np(grad).astype(np.complex128)
    assert rel(b2, bo) < FP32_BOUND
    assert np.linalg.norm(g - go) < FP32_BOUND * np.linalg.norm(go)


@pytest.fixture(scope="module")
def field16():
    U = generate.random_field((32, 16, 16, 16), 0.3, 2)
    return U, oracle.magnetic(U, parallel=True), oracle.loop5_energy_force(U, oracle.B2_PLANES)


@pytest.mark.parametrize("prec", ["c64", "r12"])
def test_fp32_b2_and_gradient_within_1e6_of_oracle(field16, prec):
    """The headline's accuracy bound: FP32 B^2 and its su(3) gradient within
    1e-6 relative (gradient: relative L2 over all links) of the FP64 oracle,
    16^3 x 32, eps 0.3."""
    U, bo, go = field16
    b, g = forces.magnetic_force(GaugeField.from_array(U, prec=prec))
    g = _np(g).astype(np.complex128)
    eb = rel(b, bo)
    eg = float(np.linalg.norm(g - go) / np.linalg.norm(go))
    print(f"{prec}: B^2 rel {eb:.2e}, gradient rel L2 {eg:.2e}")
    assert eb < FP32_BOUND
    assert eg < FP32_BOUND


def test_config1_size_haar_field():
    """32^3 x 64 Haar-random field: FP64 plaquettes, Polyakov, B^2 and u0
    against the oracle to 1e-12; FP32 B^2 within the 1e-6 bound."""
    dims = (64, 32, 32, 32)
    U = generate.haar_field(dims, 11)
    f = GaugeField.from_array(U)
    for r in ((1, 4, 4), (2, 4, 4), (1, 1, 4)):
        s, n, _ = G.plaquette(f, *r)
        so, no = oracle.genplaquette(U, *r, parallel=True)
        assert n == no and abs(s - so) < 1e-12 * n, r  # Haar sums cancel: bound per plaquette
    s, n, _ = G.polyakov(f)
    so, no = oracle.polyakov(U)
    assert n == no and abs(s - so) < 1e-12 * n
    bo = oracle.magnetic(U, parallel=True)
    assert rel(G.magnetic(f), bo) < 1e-12
    a, b = G.uzerobar(f), oracle.uzerobar(U)
    assert np.array_equal(np.isnan(a), np.isnan(b))  # a negative mean plaquette has no real root: NaN on both sides
    ok = ~np.isnan(b)
    assert not ok.any() or np.abs(a[ok] - b[ok]).max() < 1e-12
    for prec in ("c64", "r12"):
        assert rel(G.magnetic(GaugeField.from_array(f, prec=prec)), bo) < FP32_BOUND, prec
