"""CPU oracle for the FLUE gluonic-observable path (test infrastructure only).

Only the test-suite, ``__graft_entry__.smoke()`` and the CPU-baseline leg of
``bench.py`` may import this package, and only as the checker: the product
library (``flue_gb300``) never imports it.

``flue_oracle.c`` restates ``src/wloops.F90``, ``src/SU3MatrixOps.f90`` and
``FixSU3Matrix`` (``src/gaugeIO/ILDG_bin.f90:108-159``) line by line in FP64.
Parity against the reference's own outputs is unpinned (no Fortran compiler
exists on any machine this project runs on and the reference ships no golden
vectors); the routines are pinned to analytic known answers instead
(``tests/golden``).

All fields are numpy ``complex128`` arrays indexed ``data[t,x,y,z,mu,a,b]``
(any memory order; they are handed to C in the reference's Fortran order).
Directions, coordinates and path entries are 1-based like the reference's.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
import threading

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_SRC = os.path.join(_HERE, "flue_oracle.c")
_LIB = os.path.join(_HERE, "liboracle.so")
_lock = threading.Lock()
_lib = None

CFLAGS = ["-O2", "-fPIC", "-shared", "-fopenmp", "-ffp-contract=off", "-std=gnu11"]


def build(force: bool = False) -> str:
    """Compile ``flue_oracle.c`` into ``oracle/liboracle.so`` with gcc."""
    if force or not os.path.exists(_LIB) or os.path.getmtime(_LIB) < os.path.getmtime(_SRC):
        tmp = _LIB + f".tmp{os.getpid()}"
        subprocess.check_call(["gcc", *CFLAGS, "-o", tmp, _SRC, "-lm"])
        os.replace(tmp, _LIB)
    return _LIB


def lib():
    global _lib
    with _lock:
        if _lib is None:
            build()
            L = ctypes.CDLL(_LIB)
            P = ctypes.c_void_p
            I = ctypes.c_int
            D = ctypes.c_double
            sig = {
                "oracle_num_threads": ([], I),
                "oracle_multiplymatmat": ([P, P, P], None),
                "oracle_multiplymatdagmatdag": ([P, P, P], None),
                "oracle_genericpath": ([P, I, I, I, I, P, P, I, P], None),
                "oracle_genericpath_all": ([P, I, I, I, I, P, I, P], None),
                "oracle_genplaquette": ([P, I, I, I, I, I, I, I, I, P, P], None),
                "oracle_plaquette": ([P, I, I, I, I, I, I, I, P, P], None),
                "oracle_polyakov": ([P, I, I, I, I, P, P], I),
                "oracle_wmunu": ([P, I, I, I, I, I, I, I, I, I], D),
                "oracle_wmunutau": ([P, I, I, I, I, I, I, I, I, I], D),
                "oracle_clover": ([P, I, I, I, I, I, I, P], None),
                "oracle_loop5": ([P, I, I, I, I, I, I, P], None),
                "oracle_magnetic": ([P, I, I, I, I, I], D),
                "oracle_loop5_energy": ([P, I, I, I, I, P, I], D),
                "oracle_magnetic_slab": ([P, I, I, I, I, I, I], D),
                "oracle_fixsu3matrix": ([P], None),
                "oracle_fixsu3_field": ([P, I, I, I, I], None),
                "oracle_uzerobar": ([P, I, I, I, I, P, P], None),
                "oracle_plaquette_staple_force": ([P, I, I, I, I, P], None),
                "oracle_loop5_energy_force": ([P, I, I, I, I, P, I, P], None),
            }
            for name, (args, res) in sig.items():
                fn = getattr(L, name)
                fn.argtypes = args
                fn.restype = res
            _lib = L
    return _lib


# ---------------------------------------------------------------------------
# helpers
# ---------------------------------------------------------------------------
def _fortran_field(data) -> np.ndarray:
    a = np.asarray(data)
    if a.ndim != 7 or a.shape[4:] != (4, 3, 3):
        raise ValueError(f"gauge field must have shape (NT,NX,NY,NZ,4,3,3), got {a.shape}")
    return np.asfortranarray(a, dtype=np.complex128)


def _dims(a):
    return int(a.shape[0]), int(a.shape[1]), int(a.shape[2]), int(a.shape[3])


def _ptr(a: np.ndarray):
    return a.ctypes.data_as(ctypes.c_void_p)


def num_threads() -> int:
    return lib().oracle_num_threads()


# ---------------------------------------------------------------------------
# reference-shaped API (f2py conventions: intent(out) values returned)
# ---------------------------------------------------------------------------
def multiplymatmat(left, right):
    l = np.asfortranarray(left, dtype=np.complex128)
    r = np.asfortranarray(right, dtype=np.complex128)
    o = np.zeros((3, 3), dtype=np.complex128, order="F")
    lib().oracle_multiplymatmat(_ptr(o), _ptr(l), _ptr(r))
    return o


def multiplymatdagmatdag(left, right):
    l = np.asfortranarray(left, dtype=np.complex128)
    r = np.asfortranarray(right, dtype=np.complex128)
    o = np.zeros((3, 3), dtype=np.complex128, order="F")
    lib().oracle_multiplymatdagmatdag(_ptr(o), _ptr(l), _ptr(r))
    return o


def genericpath(data, coordbase, path):
    a = _fortran_field(data)
    cb = np.ascontiguousarray(coordbase, dtype=np.int32)
    p = np.ascontiguousarray(path, dtype=np.int32)
    o = np.zeros((3, 3), dtype=np.complex128, order="F")
    lib().oracle_genericpath(_ptr(a), *_dims(a), _ptr(cb), _ptr(p), int(p.size), _ptr(o))
    return o


def genericpath_all(data, path):
    a = _fortran_field(data)
    p = np.ascontiguousarray(path, dtype=np.int32)
    o = np.zeros(a.shape[:4] + (3, 3), dtype=np.complex128, order="F")
    lib().oracle_genericpath_all(_ptr(a), *_dims(a), _ptr(p), int(p.size), _ptr(o))
    return o


def genplaquette(data, mustart, muend, nuend, parallel=False):
    a = _fortran_field(data)
    s = ctypes.c_double()
    n = ctypes.c_int64()
    lib().oracle_genplaquette(_ptr(a), *_dims(a), mustart, muend, nuend, int(bool(parallel)), ctypes.byref(s), ctypes.byref(n))
    return s.value, n.value


def plaquette(data, mustart, muend, nuend):
    a = _fortran_field(data)
    s = ctypes.c_double()
    n = ctypes.c_int64()
    lib().oracle_plaquette(_ptr(a), *_dims(a), mustart, muend, nuend, ctypes.byref(s), ctypes.byref(n))
    return s.value, n.value


def polyakov(data):
    a = _fortran_field(data)
    s = ctypes.c_double()
    n = ctypes.c_int64()
    rc = lib().oracle_polyakov(_ptr(a), *_dims(a), ctypes.byref(s), ctypes.byref(n))
    if rc != 0:
        raise ValueError("polyakov: the reference defines the loop only for NT >= 3")
    return s.value, n.value


def wmunu(data, mu, nu, nmu, nnu, parallel=False):
    a = _fortran_field(data)
    return lib().oracle_wmunu(_ptr(a), *_dims(a), mu, nu, nmu, nnu, int(bool(parallel)))


def wmunutau(data, tau, mu, nu, nmu, nnu):
    a = _fortran_field(data)
    return lib().oracle_wmunutau(_ptr(a), *_dims(a), tau, mu, nu, nmu, nnu)


def cloverloopmunucoord(data, mu, nu):
    a = _fortran_field(data)
    o = np.zeros(a.shape[:4] + (3, 3), dtype=np.complex128, order="F")
    lib().oracle_clover(_ptr(a), *_dims(a), mu, nu, _ptr(o))
    return o


def loop5munucoord(data, mu, nu):
    a = _fortran_field(data)
    o = np.zeros(a.shape[:4] + (3, 3), dtype=np.complex128, order="F")
    lib().oracle_loop5(_ptr(a), *_dims(a), mu, nu, _ptr(o))
    return o


def magnetic(data, parallel=False):
    a = _fortran_field(data)
    return lib().oracle_magnetic(_ptr(a), *_dims(a), int(bool(parallel)))


def magnetic_slab(data, t_begin, t_end):
    """Raw sum of -Re Tr(F F) of magnetic() over the time slices
    t_begin..t_end (1-based, inclusive) of the full field (OpenMP)."""
    a = _fortran_field(data)
    return lib().oracle_magnetic_slab(_ptr(a), *_dims(a), int(t_begin), int(t_end))


B2_PLANES = ((3, 2), (2, 4), (4, 3))
ALL_PLANES = ((1, 2), (1, 3), (1, 4), (2, 3), (2, 4), (3, 4))


def loop5_energy(data, planes=B2_PLANES):
    a = _fortran_field(data)
    p = np.ascontiguousarray(np.asarray(planes, dtype=np.int32).reshape(-1))
    return lib().oracle_loop5_energy(_ptr(a), *_dims(a), _ptr(p), len(planes))


def fixsu3matrix(u):
    m = np.array(u, dtype=np.complex128, order="F", copy=True)
    lib().oracle_fixsu3matrix(_ptr(m))
    return m


def fixsu3_field(data):
    a = np.array(_fortran_field(data), order="F", copy=True)
    lib().oracle_fixsu3_field(_ptr(a), *_dims(a))
    return a


def uzerobar(data, g=None):
    a = _fortran_field(data)
    out = np.zeros(6, dtype=np.float64)
    gp = None
    if g is not None:
        gg = np.asfortranarray(g, dtype=np.complex128)
        if gg.shape != a.shape[:4] + (3, 3):
            raise ValueError("gauge transformation must have shape (NT,NX,NY,NZ,3,3)")
        gp = _ptr(gg)
    lib().oracle_uzerobar(_ptr(a), *_dims(a), gp, _ptr(out))
    return out


def plaquette_staple_force(data):
    a = _fortran_field(data)
    o = np.zeros(a.shape, dtype=np.complex128, order="F")
    lib().oracle_plaquette_staple_force(_ptr(a), *_dims(a), _ptr(o))
    return o


def loop5_energy_force(data, planes=B2_PLANES):
    a = _fortran_field(data)
    p = np.ascontiguousarray(np.asarray(planes, dtype=np.int32).reshape(-1))
    o = np.zeros(a.shape, dtype=np.complex128, order="F")
    lib().oracle_loop5_energy_force(_ptr(a), *_dims(a), _ptr(p), len(planes), _ptr(o))
    return o
