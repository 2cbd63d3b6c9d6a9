"""Smallest lattices: extents of 1 and 2 (every stencil wraps onto itself,
through the general wrap path) for B^2 and its gradient, the 5-loop F, the
plaquette ranges, the Polyakov loop, the W_munu table and the gluon
propagator, against the oracles in FP64."""
import numpy as np
import pytest

import oracle
from flue_gb300 import forces, generate, gluonCalc as G, gluonProp
from oracle import propagator as P

pytestmark = pytest.mark.gpu

DIMS = [(3, 1, 2, 2), (4, 2, 1, 3), (2, 3, 2, 1), (1, 2, 2, 2)]


@pytest.fixture(scope="module", params=range(len(DIMS)))
def U(request):
    return generate.random_field(DIMS[request.param], 0.6, 40 + request.param)


def test_b2_force_small_extents(U):
    b, g = forces.magnetic_force(U)
    assert abs(b - oracle.magnetic(U)) < 1e-12 * max(1.0, abs(b))
    go = oracle.loop5_energy_force(U, oracle.B2_PLANES)
    gn = g.detach().cpu().numpy() if hasattr(g, "detach") else g
    assert np.abs(gn - go).max() < 1e-11 * max(1.0, np.abs(go).max())


def test_fmunu_and_plaquettes_small_extents(U):
    for mu, nu in ((3, 2), (1, 4)):
        assert np.abs(G.loop5munucoord(U, mu, nu) - oracle.loop5munucoord(U, mu, nu)).max() < 1e-12
    for rng in ((1, 4, 4), (2, 4, 4), (1, 1, 4)):
        s, n, _ = G.plaquette(U, *rng)
        so, no = oracle.plaquette(U, *rng)
        assert n == no and abs(s - so) < 1e-12 * max(1.0, abs(so))
    if U.shape[0] >= 3:
        assert abs(G.polyakov(U)[0] - oracle.polyakov(U)[0]) < 1e-12 * U[0, ..., 0, 0, 0].size


def test_wmunu_table_and_propagator_small_extents(U):
    tab = G.wmunu_table(U, 2, 4, 3, 3)
    for r in range(3):
        for t in range(3):
            assert abs(tab[r, t] - oracle.wmunu(U, 2, 4, r + 1, t + 1)) < 1e-12
    D = gluonProp.scalar_gluon_prop(U, 1.4, 0)
    Dr = P.gluon_propagator(U, 1.4, 0)
    assert np.abs(D - Dr).max() < 1e-12 * np.abs(Dr).max()


@pytest.mark.parametrize("prec", ["c128", "c64", "r12"])
def test_nan_links_propagate_and_leave_the_library_usable(prec):
    """A NaN link makes B^2, the plaquette and the nearby gradient NaN (no
    call fails); the next calls on a clean field give the clean results."""
    from flue_gb300.field import GaugeField

    U = generate.random_field((4, 4, 4, 4), 0.4, 50)
    clean = forces.magnetic_force(GaugeField.from_array(U, prec=prec))[0]
    bad = U.copy()
    bad[1, 2, 0, 3, 2, 0, 1] = np.nan
    b, g = forces.magnetic_force(GaugeField.from_array(bad, prec=prec))
    gn = g.detach().cpu().numpy()
    assert np.isnan(b) and np.isnan(gn).any() and np.isfinite(gn).any()
    assert np.isnan(G.plaquette(GaugeField.from_array(bad, prec=prec), 1, 4, 4)[0])
    again = forces.magnetic_force(GaugeField.from_array(U, prec=prec))[0]
    assert again == clean


def test_workspace_cache_is_bounded_across_streams():
    """Calls on many streams get their own scratch; the cache keeps at most
    MAX_ENTRIES buffers and every call still gives the same B^2."""
    import torch

    from flue_gb300.field import GaugeField, Workspace

    f = GaugeField.from_array(generate.random_field((4, 4, 4, 4), 0.4, 51), prec="r12")
    ref = G.magnetic(f)
    streams = [torch.cuda.Stream() for _ in range(3 * Workspace.MAX_ENTRIES)]
    for s in streams:
        with torch.cuda.stream(s):
            assert G.magnetic(f) == ref
    torch.cuda.synchronize()
    assert len(Workspace._bufs) <= Workspace.MAX_ENTRIES


@pytest.mark.parametrize("dims", [(1, 4, 4, 4), (2, 3, 4, 5), (3, 2, 2, 2)])
@pytest.mark.parametrize("slabs", ["1", "99"])
def test_host_buffer_force_small_extents(dims, slabs, monkeypatch):
    """flue_magnetic_force_c on lattices with extents 1-3, as one pass and as
    one-slice slabs (FLUE_SLABS above NT): the device path's B^2 and gradient."""
    import ctypes

    import torch

    from flue_gb300 import _lib
    from flue_gb300.field import GaugeField

    U = generate.random_field(dims, 0.5, 52)
    b0, g0 = forces.magnetic_force(GaugeField.from_array(U, prec="c64"))
    g0 = g0.detach().cpu().numpy()
    host = torch.as_tensor(np.asfortranarray(U.astype(np.complex64))).permute(6, 5, 4, 3, 2, 1, 0)
    host = host.contiguous().pin_memory()
    grad = torch.full_like(host, float("nan")).pin_memory()
    monkeypatch.setenv("FLUE_SLABS", slabs)
    L = _lib.load()
    b = ctypes.c_double()
    rc = L.flue_magnetic_force_c(ctypes.c_void_p(host.data_ptr()), _lib.C64, *dims, _lib.C64, _lib.FORCE_LIE,
                                 ctypes.byref(b), ctypes.c_void_p(grad.data_ptr()))
    assert rc == 0, L.flue_last_error_detail()
    g = grad.permute(6, 5, 4, 3, 2, 1, 0).numpy()
    assert np.isfinite(g).all()
    assert abs(b.value - b0) < 1e-12 * max(1.0, abs(b0))
    assert np.abs(g - g0).max() < 1e-6 * np.abs(g0).max()
