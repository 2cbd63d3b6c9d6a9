"""Wilson flow: the GPU RK3 step against a numpy RK3 built from the oracle's
analytic staple force and eigen-decomposition exponentials (FP64)."""
import numpy as np
import pytest

import oracle
from flue_gb300 import flow, generate
from flue_gb300.field import GaugeField
from tests import np_flue

pytestmark = pytest.mark.gpu


def _np_rk3(U, eps, nsteps):
    """Luescher RK3 with Z = 2 G (G = oracle staple force of sum Re Tr P)."""
    W = U.copy()
    for _ in range(nsteps):
        Z0 = eps * 2 * oracle.plaquette_staple_force(W)
        W1 = np_flue.expm_su3(0.25 * Z0) @ W
        Z1 = eps * 2 * oracle.plaquette_staple_force(np.asfortranarray(W1))
        W2 = np_flue.expm_su3(8 / 9 * Z1 - 17 / 36 * Z0) @ W1
        Z2 = eps * 2 * oracle.plaquette_staple_force(np.asfortranarray(W2))
        W = np.asfortranarray(np_flue.expm_su3(0.75 * Z2 - 8 / 9 * Z1 + 17 / 36 * Z0) @ W2)
    return W


# eps 0.2: |X|_F reaches ~1, so the exponential's scale-and-square branch runs
@pytest.mark.parametrize("eps,nsteps", [(0.02, 3), (0.2, 1)])
def test_rk3_step_matches_numpy(eps, nsteps):
    U = generate.random_field((4, 4, 4, 4), 0.5, 3)
    f = GaugeField.from_array(U)
    for _ in range(nsteps):
        flow.wflow_step(f, eps)
    ref = _np_rk3(U, eps, nsteps)
    assert np.abs(f.to_numpy() - ref).max() < 1e-12


def test_flow_smooths_and_records():
    U = generate.random_field((6, 6, 6, 6), 0.5, 4)
    f, recs = flow.wilson_flow(U, eps=0.02, tmax=0.4, measure_every=0.1)
    ts = [r["t"] for r in recs]
    assert np.allclose(ts, [0.0, 0.1, 0.2, 0.3, 0.4])
    plaq = [r["plaq"] for r in recs]
    b2 = [r["b2"] for r in recs]
    assert all(b > a for a, b in zip(plaq, plaq[1:]))
    assert all(b < a for a, b in zip(b2, b2[1:]))
    # links stay unitary
    V = f.to_numpy()
    assert np.abs(V @ np_flue.dag(V) - np.eye(3)).max() < 1e-12


def test_flow_fp32_tracks_fp64():
    U = generate.random_field((6, 6, 6, 6), 0.4, 5)
    _, r64 = flow.wilson_flow(U, eps=0.02, tmax=0.2, measure_every=0.1)
    _, r32 = flow.wilson_flow(GaugeField.from_array(U, prec="c64"), eps=0.02, tmax=0.2, measure_every=0.1)
    for a, b in zip(r64, r32):
        assert abs(a["plaq"] - b["plaq"]) < 1e-6
        assert abs(a["b2"] - b["b2"]) / a["b2"] < 1e-5


def test_fp32_flow_no_drift():
    """200 RK3 steps of 0.01 in FP32 (compensated reunitarisation) stay on the
    FP64 trajectory: B^2 and the plaquette to ~1e-7 relative."""
    U = generate.random_field((8, 8, 8, 8), 0.3, 6)
    _, r64 = flow.wilson_flow(U, eps=0.01, tmax=2.0, measure_every=1.0)
    _, r32 = flow.wilson_flow(GaugeField.from_array(U, prec="c64"), eps=0.01, tmax=2.0, measure_every=1.0)
    for a, b in zip(r64, r32):
        assert abs(a["b2"] - b["b2"]) / a["b2"] < 1e-6, (a, b)
        assert abs(a["plaq"] - b["plaq"]) < 1e-7, (a, b)


def test_flow_checkpoint_resume(tmp_path):
    """A flow stopped at t = 0.1 and continued from its checkpoint to t = 0.2
    gives bitwise the links and records of the uninterrupted flow."""
    U = generate.random_field((4, 4, 6, 4), 0.4, 8)
    ck = str(tmp_path / "flow.pt")
    full, r_full = flow.wilson_flow(U, eps=0.02, tmax=0.2, measure_every=0.05)
    flow.wilson_flow(U, eps=0.02, tmax=0.1, measure_every=0.05, checkpoint=ck)  # "interrupted" at t = 0.1
    resumed, r_res = flow.wilson_flow(U, eps=0.02, tmax=0.2, measure_every=0.05, checkpoint=ck)
    assert np.array_equal(resumed.to_numpy(), full.to_numpy())
    assert r_res == r_full
    with pytest.raises(ValueError):
        flow.wilson_flow(U, eps=0.01, tmax=0.2, checkpoint=ck)
