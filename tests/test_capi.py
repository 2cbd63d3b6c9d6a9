"""The C-ABI library builds, loads without a GPU and exports every symbol the
public header declares; argument validation answers before touching CUDA."""
import ctypes
import os
import re

import pytest

from flue_gb300 import _lib

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "flue_gb300.h")


def header_functions():
    txt = open(HEADER).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    names = re.findall(r"\b(flue_[a-z0-9_]+)\s*\(", txt)
    return sorted(set(names))


def test_header_declares_the_reference_boundary():
    names = header_functions()
    for must in ("flue_plaquette_c", "flue_genplaquette_c", "flue_polyakov_c", "flue_genericpath_c", "flue_wmunu_c",
                 "flue_wmunutau_c", "flue_cloverloopmunucoord_c", "flue_loop5munucoord_c", "flue_magnetic_c",
                 "flue_multiplymatmat_c", "flue_fixsu3matrix_c", "flue_uzerobar_c"):
        assert must in names


def test_library_exports_every_declared_symbol():
    L = _lib.load()
    missing = [n for n in header_functions() if not hasattr(L, n)]
    assert not missing, missing
    # the ctypes signature table covers the header
    assert set(header_functions()) <= set(_lib.SIGNATURES)


def test_host_only_queries():
    L = _lib.load()
    assert L.flue_abi_version() == 1
    assert L.flue_strerror(0) == b"ok"
    assert L.flue_field_bytes(64, 32, 32, 32, _lib.C128) == 64 * 32 ** 3 * 36 * 16
    assert L.flue_field_bytes(64, 32, 32, 32, _lib.R12) == 64 * 32 ** 3 * 12 * 16
    assert L.flue_field_bytes(0, 4, 4, 4, _lib.C128) == -1
    assert L.flue_workspace_bytes(_lib.OP_MAGNETIC_FORCE, 8, 4, 4, 4, _lib.C64) > 0
    assert L.flue_workspace_bytes(_lib.OP_MAGNETIC_FORCE, 8, 4, 4, 4, 7) == 0


def test_validation_before_cuda():
    L = _lib.load()
    f = _lib.FlueField(None, 4, 4, 4, 4, _lib.C128)
    assert L.flue_plaquette(ctypes.byref(f), 1, 4, 4, None, None, 0, None) == _lib.FLUE_ERR_ARG
    f2 = _lib.FlueField(16, 0, 4, 4, 4, _lib.C128)
    out = ctypes.c_double()
    assert L.flue_plaquette(ctypes.byref(f2), 1, 4, 4, ctypes.byref(out), None, 0, None) == _lib.FLUE_ERR_SHAPE
    f3 = _lib.FlueField(16, 4, 4, 4, 4, 9)
    assert L.flue_magnetic(ctypes.byref(f3), ctypes.byref(out), None, 0, None) == _lib.FLUE_ERR_DTYPE
    f4 = _lib.FlueField(16, 4, 4, 4, 4, _lib.C128)
    assert L.flue_wmunu(ctypes.byref(f4), 0, 5, 1, 1, 1, ctypes.byref(out), None, 0, None) == _lib.FLUE_ERR_ARG
    bad = (ctypes.c_int * 2)(1, 7)
    assert L.flue_genericpath(ctypes.byref(f4), None, bad, 2, ctypes.byref(out), None) == _lib.FLUE_ERR_ARG
    assert L.flue_magnetic_force(ctypes.byref(f4), ctypes.byref(out), None, 0, None, 0, None) == _lib.FLUE_ERR_WORKSPACE
    with pytest.raises(ValueError):
        _lib.call("flue_plaquette", ctypes.byref(f), 1, 4, 4, None, None, 0, None)


def test_jackknife_matches_definition():
    import numpy as np

    from flue_gb300 import jack

    rng = np.random.default_rng(3)
    x = rng.standard_normal(17) + 4.0
    m, e = jack.mean_and_error(x)
    assert abs(m - x.mean()) < 1e-14
    # first-order jackknife error = sqrt((n-1)/n sum (theta_i - theta_bar)^2) = std/sqrt(n) for the mean
    assert abs(e - x.std(ddof=1) / np.sqrt(x.size)) < 1e-12
    c2 = jack.complement(x, (3,))
    assert abs(c2[0] - (x.sum() - x[3] - x[0]) / (x.size - 2)) < 1e-14
