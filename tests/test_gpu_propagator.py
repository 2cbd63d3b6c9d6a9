"""Gluon propagator and gauge transformation on the GPU against the numpy
oracle (oracle/propagator.py): FP64 fields to 1e-12, FP32 (c64, r12) to
1e-5 of the largest D; odd and even extents (cuFFT's non-power-of-two
paths), anisotropy and spatial-only sums; the closed-form single mode; the
host-buffer entry; gauge transformations against numpy products."""
import numpy as np
import pytest
import torch

from flue_gb300 import generate, gluonProp
from flue_gb300.field import GaugeField
from oracle import propagator as P
from tests.test_propagator import _abelian

pytestmark = pytest.mark.gpu


def _rel(a, b):
    return np.abs(np.asarray(a) - np.asarray(b)).max() / np.abs(np.asarray(b)).max()


@pytest.mark.parametrize("dims", [(8, 4, 4, 4), (5, 3, 4, 6), (6, 5, 2, 3)])
@pytest.mark.parametrize("xi,mu_start", [(1.0, 0), (2.5, 0), (1.0, 1)])
def test_propagator_fp64_vs_oracle(dims, xi, mu_start):
    U = generate.random_field(dims, 0.5, 11)
    D = gluonProp.scalar_gluon_prop(U, xi, mu_start)
    assert D.shape == dims and D.dtype == np.float64
    assert _rel(D, P.gluon_propagator(U, xi, mu_start)) < 1e-12


@pytest.mark.parametrize("prec", ["c64", "r12"])
def test_propagator_fp32_vs_oracle(prec):
    U = generate.random_field((8, 6, 4, 5), 0.4, 12)
    D = gluonProp.scalar_gluon_prop(GaugeField.from_array(U, prec=prec), 1.3, 0)
    assert _rel(D.cpu().numpy(), P.gluon_propagator(U, 1.3, 0)) < 1e-5


def test_single_mode_on_gpu():
    dims = (6, 4, 5, 4)
    n = np.array([1, 2, 0, 1])
    grids = np.meshgrid(*[np.arange(k) for k in dims], indexing="ij")
    phase = sum(2 * np.pi * n[d] * grids[d] / dims[d] for d in range(4))
    theta = np.zeros(dims + (4,))
    theta[..., 2] = np.arcsin(0.4 * np.cos(phase))
    D = gluonProp.scalar_gluon_prop(_abelian(theta))
    V = np.prod(dims)
    expect = (0.4 * V) ** 2 / (8 * 3 * V)
    kp, km = tuple(n % np.array(dims)), tuple((-n) % np.array(dims))
    assert abs(D[kp] - expect) < 1e-12 * expect and abs(D[km] - expect) < 1e-12 * expect
    D[kp] = D[km] = 0
    assert np.abs(D).max() < 1e-12 * expect
    # positive octant: calc_mom_space_scalarD's (0:NT/2, 0:NS/2, ...) range
    assert gluonProp.positive_octant(D).shape == (4, 3, 3, 3)


def test_host_entry_scalargluonprop():
    U = generate.random_field((6, 4, 4, 4), 0.5, 13)
    assert _rel(gluonProp.scalargluonprop(U, 1.5), P.gluon_propagator(U, 1.5, 0)) < 1e-12


@pytest.mark.parametrize("prec,gdt,tol", [("c128", np.complex128, 1e-13), ("c64", np.complex64, 3e-6),
                                          ("r12", np.complex128, 3e-6)])
def test_gauge_transform(prec, gdt, tol):
    dims = (4, 3, 4, 5)
    U = generate.random_field(dims, 0.6, 14)
    G = generate.random_gauge_transform(dims, 15)
    f = GaugeField.from_array(U, prec=prec)
    gluonProp.gauge_transform(f, G.astype(gdt))
    Gp = [np.roll(G, -1, axis=mu) for mu in range(4)]
    ref = np.stack([np.einsum("...ij,...jk,...lk->...il", G, U[..., mu, :, :], np.conj(Gp[mu]))
                    for mu in range(4)], axis=4)
    assert np.abs(f.to_numpy() - ref).max() < tol


def test_global_gauge_rotation_leaves_propagator():
    U = generate.random_field((6, 4, 4, 4), 0.5, 16)
    f = GaugeField.from_array(U)
    D0 = gluonProp.scalar_gluon_prop(f).cpu().numpy()
    g = generate.random_gauge_transform((1, 1, 1, 1), 17)[0, 0, 0, 0]
    G = np.broadcast_to(g, (6, 4, 4, 4, 3, 3)).copy()
    gluonProp.gauge_transform(f, G)
    assert _rel(gluonProp.scalar_gluon_prop(f).cpu().numpy(), D0) < 1e-12
