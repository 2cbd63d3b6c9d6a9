"""GPU parity: every observable of the CUDA path against the CPU oracle on the
same seeded fields.  FP64 (c128) results must agree to 1e-12 relative (sums)
or 1e-12 absolute (matrix elements, which are O(1)); FP32 (c64 / r12) results
are held to the FP32 bounds stated per test."""
import ctypes
import json
import os

import numpy as np
import pytest
import torch

import oracle
from flue_gb300 import _lib, generate, gluonCalc as G
from flue_gb300.field import GaugeField
from tests.golden.make_golden import abelian_field

pytestmark = pytest.mark.gpu
GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")

# lattices: tiny / odd extents catch wrap-around and tiling bugs
CASES = [((4, 4, 4, 4), 0.3, 1), ((5, 3, 4, 6), 0.5, 2), ((3, 2, 3, 2), 0.8, 3), ((8, 6, 6, 6), "haar", 4)]


def _field(case):
    dims, eps, seed = case
    return generate.haar_field(dims, seed) if eps == "haar" else generate.random_field(dims, eps, seed)


@pytest.fixture(scope="module", params=range(len(CASES)))
def U(request):
    return _field(CASES[request.param])


def rel(a, b):
    return abs(a - b) / max(abs(b), 1e-300)


def test_plaquette_fp64(U):
    for r in ((1, 4, 4), (2, 4, 4), (1, 1, 4), (2, 3, 4), (3, 3, 3)):
        s, n, t = G.plaquette(U, *r)
        so, no = oracle.plaquette(U, *r)
        assert n == no
        if no:
            assert rel(s, so) < 1e-12, r
        assert t >= 0
        s2, n2, _ = G.genplaquette(U, *r)
        assert s2 == s and n2 == n


def test_polyakov_fp64(U):
    if U.shape[0] < 3:
        pytest.skip("the reference defines the Polyakov loop for NT >= 3")
    s, n, _ = G.polyakov(U)
    so, no = oracle.polyakov(U)
    assert n == no
    assert abs(s - so) < 1e-12 * max(1.0, n)


def test_genericpath_fp64(U):
    for path in ([1, 2, -1, -2], [2, 2, 3, -4, -2, 1, 1, -3], [-1, -1, 4, 3, 3, 3, -2]):
        a = G.genericpath_all(U, path)
        b = oracle.genericpath_all(U, path)
        assert np.abs(a - b).max() < 1e-12
        cb = [1 + (k + 1) % U.shape[k] for k in range(4)]
        g = G.genericpath(U, cb, path)
        assert np.abs(g - oracle.genericpath(U, cb, path)).max() < 1e-12


def test_wilson_loops_fp64(U):
    for (mu, nu, r, t) in ((2, 3, 1, 1), (1, 4, 2, 3), (3, 2, 3, 2), (4, 1, 1, 5)):
        assert abs(G.wmunu(U, mu, nu, r, t) - oracle.wmunu(U, mu, nu, r, t)) < 1e-12
    tau = U.shape[0]
    assert abs(G.wmunutau(U, tau, 2, 4, 2, 1) - oracle.wmunutau(U, tau, 2, 4, 2, 1)) < 1e-12
    tab = G.wmunu_table(U, 2, 3, 3, 2)
    for r in range(3):
        for t in range(2):
            assert abs(tab[r, t] - oracle.wmunu(U, 2, 3, r + 1, t + 1)) < 1e-12


def test_fmunu_fp64(U):
    for mu, nu in ((3, 2), (1, 4), (2, 4)):
        a = G.loop5munucoord(U, mu, nu)
        b = oracle.loop5munucoord(U, mu, nu)
        assert np.abs(a - b).max() < 1e-12
        c = G.cloverloopmunucoord(U, mu, nu)
        d = oracle.cloverloopmunucoord(U, mu, nu)
        assert np.abs(c - d).max() < 1e-12


def test_magnetic_fp64(U):
    assert rel(G.magnetic(U), oracle.magnetic(U)) < 1e-12


def test_uzerobar_fp64(U):
    g = generate.random_gauge_transform(U.shape[:4], 8)
    a = G.uzerobar(U, g)
    b = oracle.uzerobar(U, g)
    # Haar fields can have <Re Tr P> < 0: both sides give NaN there
    assert np.array_equal(np.isnan(a), np.isnan(b))
    ok = ~np.isnan(b)
    assert np.abs(a[ok] - b[ok]).max() < 1e-12


def test_su3_helpers():
    rng = np.random.default_rng(5)
    a = rng.standard_normal((7, 3, 3)) + 1j * rng.standard_normal((7, 3, 3))
    b = rng.standard_normal((7, 3, 3)) + 1j * rng.standard_normal((7, 3, 3))
    mm = G.multiplymatmat(a, b)
    dd = G.multiplymatdagmatdag(a, b)
    for k in range(7):
        assert np.abs(mm[k] - oracle.multiplymatmat(a[k], b[k])).max() < 1e-13
        assert np.abs(dd[k] - oracle.multiplymatdagmatdag(a[k], b[k])).max() < 1e-13
    f = G.fixsu3matrix(a)
    for k in range(7):
        assert np.abs(f[k] - oracle.fixsu3matrix(a[k])).max() < 1e-13


def test_abelian_known_answers_on_gpu():
    kats = json.load(open(os.path.join(GOLD, "abelian_kat.json")))
    for kat in kats:
        U = abelian_field(kat["case"])
        ex = kat["expected"]
        assert rel(G.plaquette(U, 1, 4, 4)[0], ex["plaq_all"]) < 1e-13
        assert rel(G.plaquette(U, 2, 4, 4)[0], ex["plaq_spatial"]) < 1e-13
        assert abs(G.polyakov(U)[0] - ex["polyakov"]) < 1e-10
        assert abs(G.wmunu(U, 2, 3, 2, 3) - ex["wmunu_23"]["2,3"]) < 1e-12
        f5 = G.loop5munucoord(U, 2, 3)
        for a in range(3):
            assert np.allclose(f5[..., a, a], 1j * ex["loop5_diag_im"][a], atol=1e-13)
        assert abs(G.magnetic(U) - ex["magnetic"]) < 1e-12


def test_cold_field_exact():
    U = generate.cold_field((4, 4, 4, 8))
    V = 4 * 4 * 4 * 8
    assert G.plaquette(U, 1, 4, 4)[:2] == (18.0 * V, 6 * V)
    assert G.polyakov(U)[:2] == (3.0 * 128, 128)
    assert G.magnetic(U) == 0.0


# ---------------------------------------------------------------------------
# device-resident field, layouts and precisions
# ---------------------------------------------------------------------------
def test_layouts_roundtrip():
    U = _field(CASES[1])
    f = GaugeField.from_array(U)  # Fortran order -> zero re-layout
    assert np.array_equal(f.to_numpy(), U)
    c = np.ascontiguousarray(U)  # C order -> pack kernel
    f2 = GaugeField.from_array(torch.as_tensor(c).cuda())
    assert np.array_equal(f2.to_numpy(), U)
    r = GaugeField.from_array(U, prec="r12")
    back = r.to_numpy()
    assert np.abs(back - U).max() < 5e-7


# FP32 bounds (link products in FP32, sums in FP64), each a few times the
# largest error measured on the GB300 over the parity lattices (4^4 to 16x8^3,
# eps 0.3 to 0.8 and Haar, c64 and r12): B^2 3.7e-8 relative, gradient
# 3.0e-7 relative L2 and 4.7e-7 of its largest element, plaquette 2.0e-8 and
# Polyakov 2.7e-8 per term, genericPath 4.6e-7, W loops 9.3e-8, clover and
# 5-loop F 3.2e-7 and 3.6e-7 of their largest element.
FP32_B2 = 1e-6  # the headline's bound for B^2 and its gradient (relative L2)
FP32_PER_TERM = 2e-7
FP32_MATRIX = 2e-6


@pytest.mark.parametrize("prec", ["c64", "r12"])
def test_fp32_observables(prec):
    U = _field(((8, 4, 6, 4), 0.3, 9))
    f = GaugeField.from_array(U, prec=prec)
    for r in ((1, 4, 4), (2, 4, 4), (1, 1, 4)):
        s, n, _ = G.plaquette(f, *r)
        assert abs(s - oracle.plaquette(U, *r)[0]) < FP32_PER_TERM * n
    s, n, _ = G.polyakov(f)
    assert abs(s - oracle.polyakov(U)[0]) < FP32_PER_TERM * n
    assert rel(G.magnetic(f), oracle.magnetic(U)) < FP32_B2
    a = G.loop5munucoord(f, 3, 2).cpu().numpy()
    q = oracle.loop5munucoord(U, 3, 2)
    assert np.abs(a - q).max() < FP32_MATRIX * np.abs(q).max()


def _host(x):
    return x.detach().cpu().numpy() if isinstance(x, torch.Tensor) else np.asarray(x)


@pytest.mark.parametrize("prec", ["c64", "r12"])
def test_fp32_every_observable(U, prec):
    """FP32 links (complex64 and reconstruct-12) against the FP64 oracle on
    every parity lattice (odd and tiny extents, a Haar field): bounds per
    element, absolute where sums cancel, growing with the links per loop."""
    from flue_gb300 import forces

    f = GaugeField.from_array(U, prec=prec)
    for r in ((1, 4, 4), (2, 4, 4), (1, 1, 4)):
        s, n, _ = G.plaquette(f, *r)
        so, no = oracle.plaquette(U, *r)
        assert n == no and abs(s - so) < FP32_PER_TERM * n, r
    if U.shape[0] >= 3:
        s, n, _ = G.polyakov(f)
        so, no = oracle.polyakov(U)
        assert n == no and abs(s - so) < FP32_PER_TERM * n
    for args in ((2, 3, 2, 1), (1, 4, 1, 2), (4, 2, 3, 3)):
        assert abs(G.wmunu(f, *args) - oracle.wmunu(U, *args)) < 1e-6, args
    assert abs(G.wmunutau(f, 1, 2, 4, 2, 1) - oracle.wmunutau(U, 1, 2, 4, 2, 1)) < 1e-6
    tab = _host(G.wmunu_table(f, 3, 4, 3, 2))
    for r in range(3):
        for t in range(2):
            assert abs(tab[r, t] - oracle.wmunu(U, 3, 4, r + 1, t + 1)) < 1e-6, (r, t)
    path = [2, 3, -2, 4, -3, -4, 1, -1]
    gp = _host(G.genericpath(f, [1, 1, 1, 1], path))
    assert np.abs(gp - oracle.genericpath(U, [1, 1, 1, 1], path)).max() < FP32_MATRIX
    assert np.abs(_host(G.genericpath_all(f, path)) - oracle.genericpath_all(U, path)).max() < FP32_MATRIX
    for mu, nu in ((1, 2), (3, 4)):
        co = oracle.cloverloopmunucoord(U, mu, nu)
        c = _host(G.cloverloopmunucoord(f, mu, nu))
        assert np.abs(c - co).max() < FP32_MATRIX * np.abs(co).max(), (mu, nu)
        qo = oracle.loop5munucoord(U, mu, nu)
        q = _host(G.loop5munucoord(f, mu, nu))
        assert np.abs(q - qo).max() < FP32_MATRIX * np.abs(qo).max(), (mu, nu)
    b = G.magnetic(f)
    bo = oracle.magnetic(U)
    assert rel(b, bo) < FP32_B2
    b, g = forces.magnetic_force(f)
    g = _host(g).astype(np.complex128)
    go = oracle.loop5_energy_force(U, oracle.B2_PLANES)
    assert rel(b, bo) < FP32_B2
    assert np.linalg.norm(g - go) < FP32_B2 * np.linalg.norm(go)
    assert np.abs(g - go).max() < FP32_MATRIX * np.abs(go).max()


# ---------------------------------------------------------------------------
# the host-buffer tier (reference signatures) through ctypes
# ---------------------------------------------------------------------------
def test_host_buffer_tier():
    U = _field(CASES[0])
    L = _lib.load()
    nt, nx, ny, nz = U.shape[:4]
    d = U.ctypes.data_as(ctypes.c_void_p)
    s, n, t = ctypes.c_double(), ctypes.c_int(), ctypes.c_double()
    assert L.flue_plaquette_c(d, nt, nx, ny, nz, 1, 4, 4, ctypes.byref(s), ctypes.byref(n), ctypes.byref(t)) == 0
    so, no = oracle.plaquette(U, 1, 4, 4)
    assert rel(s.value, so) < 1e-12 and n.value == no
    assert L.flue_polyakov_c(d, nt, nx, ny, nz, ctypes.byref(s), ctypes.byref(n), ctypes.byref(t)) == 0
    assert abs(s.value - oracle.polyakov(U)[0]) < 1e-12 * n.value
    b = ctypes.c_double()
    assert L.flue_magnetic_c(d, nt, nx, ny, nz, ctypes.byref(b)) == 0
    assert rel(b.value, oracle.magnetic(U)) < 1e-12
    w = ctypes.c_double()
    assert L.flue_wmunu_c(d, nt, nx, ny, nz, 2, 3, 2, 2, ctypes.byref(w)) == 0
    assert abs(w.value - oracle.wmunu(U, 2, 3, 2, 2)) < 1e-12
    assert L.flue_wmunutau_c(d, nt, nx, ny, nz, 2, 1, 3, 1, 2, ctypes.byref(w)) == 0
    assert abs(w.value - oracle.wmunutau(U, 2, 1, 3, 1, 2)) < 1e-12
    out = np.zeros((nt, nx, ny, nz, 3, 3), dtype=np.complex128, order="F")
    assert L.flue_loop5munucoord_c(d, nt, nx, ny, nz, 3, 2, out.ctypes.data_as(ctypes.c_void_p)) == 0
    assert np.abs(out - oracle.loop5munucoord(U, 3, 2)).max() < 1e-12
    assert L.flue_cloverloopmunucoord_c(d, nt, nx, ny, nz, 1, 2, out.ctypes.data_as(ctypes.c_void_p)) == 0
    assert np.abs(out - oracle.cloverloopmunucoord(U, 1, 2)).max() < 1e-12
    cb = (ctypes.c_int * 4)(2, 1, 3, 4)
    path = (ctypes.c_int * 5)(1, 3, -1, 4, -3)
    g = np.zeros((3, 3), dtype=np.complex128, order="F")
    assert L.flue_genericpath_c(d, nt, nx, ny, nz, cb, path, 5, g.ctypes.data_as(ctypes.c_void_p)) == 0
    assert np.abs(g - oracle.genericpath(U, [2, 1, 3, 4], [1, 3, -1, 4, -3])).max() < 1e-13
    a = np.asfortranarray(U[0, 0, 0, 0, 1])
    bb = np.asfortranarray(U[1, 0, 0, 0, 2])
    mm = np.zeros((3, 3), dtype=np.complex128, order="F")
    assert L.flue_multiplymatmat_c(mm.ctypes.data_as(ctypes.c_void_p), a.ctypes.data_as(ctypes.c_void_p),
                                   bb.ctypes.data_as(ctypes.c_void_p)) == 0
    assert np.abs(mm - a @ bb).max() < 1e-14
    m = np.asfortranarray(np.random.default_rng(3).standard_normal((3, 3)) * (1 + 0.5j))
    ref = oracle.fixsu3matrix(m)
    assert L.flue_fixsu3matrix_c(m.ctypes.data_as(ctypes.c_void_p)) == 0
    assert np.abs(m - ref).max() < 1e-14
    gt = generate.random_gauge_transform(U.shape[:4], 4)
    u0 = np.zeros(6)
    assert L.flue_uzerobar_c(d, nt, nx, ny, nz, gt.ctypes.data_as(ctypes.c_void_p),
                             u0.ctypes.data_as(ctypes.c_void_p)) == 0
    assert np.abs(u0 - oracle.uzerobar(U, gt)).max() < 1e-12
    # errors come back as status codes
    assert L.flue_plaquette_c(d, nt, nx, ny, nz, 0, 4, 4, ctypes.byref(s), ctypes.byref(n), ctypes.byref(t)) != 0


def test_kernel_launch_counter():
    """flue_kernel_launches counts the kernels a call runs: the plaquette is
    one reduction kernel and its finisher."""
    f = GaugeField.from_array(generate.random_field((4, 4, 4, 4), 0.3, 12))
    L = _lib.load()
    G.plaquette(f, 1, 4, 4)
    n0 = L.flue_kernel_launches()
    G.plaquette(f, 1, 4, 4)
    assert L.flue_kernel_launches() - n0 == 2


@pytest.mark.parametrize("dims,mu,nu,rmax,tmax", [((6, 4, 5, 3), 2, 3, 8, 8), ((5, 3, 4, 6), 1, 4, 7, 9),
                                                  ((4, 4, 4, 4), 4, 2, 5, 3)])
def test_wmunu_table_vs_single_loops(dims, mu, nu, rmax, tmax):
    """The table entry (lines built once per site) against one wmunu call
    per (R, T) and the oracle, R and T up to and past the extents (the walk
    wraps), FP64 to 1e-12; FP32 against FP64 to 1e-5."""
    U = generate.random_field(dims, 0.4, 31)
    tab = G.wmunu_table(U, mu, nu, rmax, tmax)
    for r in range(rmax):
        for t in range(tmax):
            single = G.wmunu(U, mu, nu, r + 1, t + 1)
            assert abs(tab[r, t] - single) < 1e-12 * max(1.0, abs(single))
    for r, t in ((0, 0), (rmax - 1, tmax - 1), (rmax // 2, 1)):
        assert abs(tab[r, t] - oracle.wmunu(U, mu, nu, r + 1, t + 1)) < 1e-12
    tab32 = G.wmunu_table(GaugeField.from_array(U, prec="r12"), mu, nu, rmax, tmax)
    assert np.abs(tab32 - tab).max() < 1e-5
