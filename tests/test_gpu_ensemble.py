"""Ensemble batching on the GPU: one persistent, graph-captured launch over
fields of uneven volume against the oracle, field by field; with many time
slabs per field (the ring of line slots reused many times over, so the
scheduler's waits are exercised) the results equal those of the default
slabs."""
import numpy as np
import pytest

import oracle
from flue_gb300 import ensemble, generate
from flue_gb300.field import GaugeField

pytestmark = pytest.mark.gpu

DIMS = [(4, 4, 4, 4), (6, 4, 4, 4), (8, 6, 6, 6), (5, 3, 4, 6), (4, 6, 6, 6), (3, 2, 3, 2)]


@pytest.fixture(scope="module")
def fields_np():
    return [generate.random_field(d, 0.4, 100 + i) for i, d in enumerate(DIMS)]


def _check(raw, fields_np, tol_sum, tol_b2):
    for row, U in zip(raw, fields_np):
        sp = oracle.plaquette(U, 2, 4, 4)[0]
        tp = oracle.plaquette(U, 1, 1, 4)[0]
        assert abs(row[0] - sp) <= tol_sum * abs(sp)
        assert abs(row[1] - tp) <= tol_sum * abs(tp)
        if U.shape[0] >= 3:
            assert abs(row[2] - oracle.polyakov(U)[0]) <= tol_sum * U[0].size / 36 * 3
        assert abs(row[4] - oracle.magnetic(U)) <= tol_b2 * abs(row[4])
        assert row[5] == np.prod(U.shape[:4])


@pytest.mark.parametrize("tile,block,bps", [(1, 128, 1), (4, 256, 2), (16, 256, 4)])
def test_ensemble_fp64_vs_oracle(fields_np, tile, block, bps):
    fs = [GaugeField.from_array(U) for U in fields_np]
    ens = ensemble.Ensemble(fs, tile=tile, block=block, blocks_per_sm=bps)
    direct = ens.run(graph=False).copy()
    graphed = ens.run(graph=True)
    again = ens.run(graph=True)
    assert np.array_equal(direct, graphed) and np.array_equal(graphed, again)
    _check(graphed, fields_np, 1e-12, 1e-12)


@pytest.mark.parametrize("prec", ["c64", "r12"])
def test_ensemble_fp32(fields_np, prec):
    fs = [GaugeField.from_array(U, prec=prec) for U in fields_np]
    raw = ensemble.Ensemble(fs, tile=2).run()
    _check(raw, fields_np, 3e-6, 1e-6)


def test_autotune_and_observables(fields_np, tmp_path, monkeypatch):
    monkeypatch.setenv("FLUE_CACHE_DIR", str(tmp_path))
    fs = [GaugeField.from_array(U) for U in fields_np]
    cands = [(1, 128, 1), (4, 256, 2)]
    best = ensemble.autotune(fs, candidates=cands)
    assert tuple(best) in cands
    assert ensemble.autotune(fs, candidates=cands) == tuple(best)  # served from the cache
    obs = ensemble.Ensemble(fs, tile=best[0], block=best[1], blocks_per_sm=best[2]).observables()
    for o, U in zip(obs, fields_np):
        s, n = oracle.plaquette(U, 1, 4, 4)
        assert abs(o["plaq"] - s / n / 3) < 1e-12


def test_mixed_precision_rejected(fields_np):
    with pytest.raises(TypeError):
        ensemble.Ensemble([GaugeField.from_array(fields_np[0]), GaugeField.from_array(fields_np[1], prec="c64")])


@pytest.mark.parametrize("prec,tol_sum,tol_b2", [("c128", 1e-12, 1e-12), ("c64", 3e-6, 1e-6), ("r12", 3e-6, 1e-6)])
def test_ensemble_pipeline_mode(fields_np, prec, tol_sum, tol_b2):
    """Pipeline mode (per-field entry points in one graph): the same outputs,
    direct and replayed bitwise equal, and the kernel-launch counter counts a
    replay as the kernels a direct evaluation launches."""
    from flue_gb300 import _lib

    fs = [GaugeField.from_array(U, prec=prec) for U in fields_np]
    ens = ensemble.Ensemble(fs, mode="pipeline")
    L = _lib.load()
    n0 = L.flue_kernel_launches()
    direct = ens.run(graph=False).copy()
    n_direct = L.flue_kernel_launches() - n0
    graphed = ens.run(graph=True)  # captures (one uncaptured evaluation first), then replays
    n1 = L.flue_kernel_launches()
    again = ens.run(graph=True)
    assert L.flue_kernel_launches() - n1 == n_direct
    assert np.array_equal(direct, graphed) and np.array_equal(graphed, again)
    _check(graphed, fields_np, tol_sum, tol_b2)
    if prec == "c128":  # the persistent kernel and the pipeline agree
        persistent = ensemble.Ensemble(fs, tile=4).run()
        assert np.allclose(persistent, graphed, rtol=1e-12, atol=0)


@pytest.mark.parametrize("prec", ["c128", "r12"])
def test_ensemble_many_slabs(fields_np, prec, monkeypatch):
    """One time slice per slab (FLUE_ENS_SLAB_SITES=1): 30 slabs through 4
    line slots, every forward task waiting on its slab's line tasks and every
    line task on the release of its slot; the same sums as the default slabs
    (FP64 summation order) and the oracle."""
    fs = [GaugeField.from_array(U, prec=prec) for U in fields_np]
    ref = ensemble.Ensemble(fs, tile=4).run()
    monkeypatch.setenv("FLUE_ENS_SLAB_SITES", "1")
    ens = ensemble.Ensemble(fs, tile=4, block=128, blocks_per_sm=1)
    for graph in (False, True, True):
        raw = ens.run(graph=graph)
        assert np.allclose(raw, ref, rtol=1e-12, atol=1e-12)
    _check(raw, fields_np, 1e-12 if prec == "c128" else 3e-6, 1e-12 if prec == "c128" else 1e-6)
