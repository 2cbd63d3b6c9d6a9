"""Bounds-checked build (the check compute-sanitizer would give, which this
pool closes): the library compiled with -DFLUE_BOUNDS_CHECK=1 into a
temporary directory, where
every link and intermediate accessor (and the raw-indexed flow, gauge and
propagator kernels) checks its indices and counts violations instead of
touching memory.  Every entry point runs on small and odd lattices in all
three precisions -- with and without time slabs, the host-buffer pipeline,
both ensemble modes, the Wilson flow and the propagator -- and no kernel may
index outside its buffers; the results agree with the normal build's."""
import ctypes
import os

import numpy as np
import pytest
import torch

from flue_gb300 import _lib, build, ensemble, flow, forces, generate, gluonCalc as G, gluonProp
from flue_gb300.field import GaugeField

pytestmark = pytest.mark.gpu

DIMS = [(4, 4, 4, 4), (5, 3, 4, 6), (3, 2, 3, 2), (1, 2, 2, 2), (8, 4, 6, 4)]
PATH = [2, 3, -2, 4, -3, -4, 1]


def _run_all(U, prec):
    f = GaugeField.from_array(U, prec=prec)
    out = [G.plaquette(f, 1, 4, 4)[0], G.polyakov(f)[0], G.wmunu(f, 2, 3, 2, 1), G.magnetic(f)]
    out.append(float(G.wmunu_table(f, 2, 4, 3, 2).sum()))
    out.append(float(np.abs(np.asarray(G.genericpath_all(f, PATH).cpu())).sum()))
    out.append(float(np.abs(np.asarray(G.loop5munucoord(f, 3, 2).cpu())).sum()))
    out.append(float(np.abs(np.asarray(G.cloverloopmunucoord(f, 1, 4).cpu())).sum()))
    b, g = forces.magnetic_force(f)
    out += [b, float(g.abs().sum())]
    e, g = forces.loop5_energy_force(f)
    out += [e, float(g.abs().sum())]
    s, g = forces.plaquette_force(f)
    out += [s, float(g.abs().sum())]
    out.append(float(gluonProp.scalar_gluon_prop(f, 1.2, 0).sum()))
    Gt = generate.random_gauge_transform(U.shape[:4], 7)
    h = f.clone()
    gluonProp.gauge_transform(h, Gt)
    out.append(G.plaquette(h, 1, 4, 4)[0])
    if prec != "r12":
        h = f.clone()
        flow.wflow_step(h, 0.02)
        out.append(G.plaquette(h, 1, 4, 4)[0])
    return np.array(out, dtype=np.float64)


@pytest.fixture(scope="module")
def checked(tmp_path_factory):
    d = tmp_path_factory.mktemp("bounds")
    path = build.build(force=True, extra_flags=["-DFLUE_BOUNDS_CHECK=1"], lib_path=str(d / "libchecked.so"),
                       build_dir=str(d / "obj"))
    L = ctypes.CDLL(path)
    for name, (args, res) in _lib.SIGNATURES.items():
        fn = getattr(L, name)
        fn.argtypes, fn.restype = args, res
    return L


def test_no_out_of_bounds_access(checked, monkeypatch):
    fields = [generate.random_field(d, 0.5, 70 + i) for i, d in enumerate(DIMS)]
    normal = {(i, p): _run_all(U, p) for i, U in enumerate(fields) for p in ("c128", "c64", "r12")}
    assert _lib.load().flue_bounds_errors() == -1  # the normal build has no checks
    saved = _lib._lib
    _lib._lib = checked
    try:
        assert checked.flue_bounds_errors() == 0
        for (i, p), ref in normal.items():
            got = _run_all(fields[i], p)
            assert checked.flue_bounds_errors() == 0, (DIMS[i], p)
            assert np.allclose(got, ref, rtol=1e-12 if p == "c128" else 1e-5, atol=0), (DIMS[i], p)
        # time slabs on several streams, the host-buffer pipeline, both ensemble modes
        monkeypatch.setenv("FLUE_SLABS", "3")
        U = fields[4]
        for p in ("c64", "r12"):
            forces.magnetic_force(GaugeField.from_array(U, prec=p))
            host = torch.as_tensor(np.asfortranarray(U.astype(np.complex64))).permute(6, 5, 4, 3, 2, 1, 0)
            host = host.contiguous().pin_memory()
            grad = torch.empty_like(host).pin_memory()
            b = ctypes.c_double()
            code = {"c64": _lib.C64, "r12": _lib.R12}[p]
            assert checked.flue_magnetic_force_c(ctypes.c_void_p(host.data_ptr()), _lib.C64, *U.shape[:4], code,
                                                 _lib.FORCE_LIE, ctypes.byref(b),
                                                 ctypes.c_void_p(grad.data_ptr())) == 0
        fs = [GaugeField.from_array(V, prec="c64") for V in fields]
        for ens in (ensemble.Ensemble(fs, tile=2), ensemble.Ensemble(fs, mode="pipeline")):
            ens.run()
            ens.close()  # with the library that created it
        assert checked.flue_bounds_errors() == 0
    finally:
        _lib._lib = saved
        os.environ.pop("FLUE_SLABS", None)
