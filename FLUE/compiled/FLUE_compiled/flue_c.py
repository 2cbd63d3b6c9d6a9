"""``flue_c``: the f2py module of c_wrapper/FLUE_c.f90, rebuilt over the C ABI
of ``libflue_gb300.so`` (include/flue_gb300.h, host-buffer tier).

f2py conventions kept (numpy.f2py ... --lower, python/meson.build:55-67):

* lower-case names;
* ``intent(in)`` arrays first, converted to Fortran-ordered complex128 /
  float64 / int32 copies when their dtype or order differ (f2py copies too);
* array extents (NT, NX, NY, NZ, NS, NQ) are inferred from the arrays and
  may be passed as trailing keywords, which must then agree;
* ``intent(out)`` values are returned -- one value alone, several as a tuple
  in declaration order; ``intent(inout)`` arrays are updated in place and
  must already be Fortran-contiguous arrays of the right dtype;
* integer directions, coordinates and path entries stay 1-based;
* a bad shape, dtype or value raises ValueError / TypeError (the Fortran
  would ``stop`` or read out of bounds; f2py raises on shape mismatches).

The routines of the reference's FLUE_c.f90 (scalargluonprop_c,
calc_mom_space_scalard_c, multiplymatmat_c, q_average_c, get_qhat_c,
cone_cut_c) keep their names and argument order.  The wloops routines of the
hot path (src/wloops.F90), which the reference has not wrapped yet, are added
under their own lower-case names (``plaquette``, ``polyakov``, ...) and, for
a wrapper following FLUE_c.f90's naming, with a ``_c`` suffix as well.
"""
from __future__ import annotations

import ctypes

import numpy as np

from flue_gb300 import _lib, gluonAna as _ana, gluonProp as _prop

__all__ = [
    "multiplymatmat_c", "scalargluonprop_c", "calc_mom_space_scalard_c", "q_average_c", "get_qhat_c", "cone_cut_c",
    "plaquette", "genplaquette", "polyakov", "genericpath", "wmunu", "wmunutau", "cloverloopmunucoord",
    "loop5munucoord", "magnetic", "magnetic_force", "uzerobar", "fixsu3matrix",
]

_VP = ctypes.c_void_p


def _p(a: np.ndarray):
    return a.ctypes.data_as(_VP)


def _field(data, nt=None, nx=None, ny=None, nz=None):
    """complex(C_DOUBLE) data(NT,NX,NY,NZ,4,3,3) (src/wloops.F90:60) as a
    Fortran-ordered complex128 array, extents checked against the keywords."""
    a = np.asarray(data)
    if a.ndim != 7 or a.shape[4:] != (4, 3, 3):
        raise ValueError(f"data must have shape (NT,NX,NY,NZ,4,3,3), got {a.shape}")
    if not np.issubdtype(a.dtype, np.number):
        raise TypeError(f"data must be numeric, got {a.dtype}")
    a = np.asfortranarray(a, dtype=np.complex128)
    dims = tuple(int(v) for v in a.shape[:4])
    for name, given, have in zip(("nt", "nx", "ny", "nz"), (nt, nx, ny, nz), dims):
        if given is not None and int(given) != have:
            raise ValueError(f"{name}={given} does not match the extent {have} of data")
    return a, dims


def _mat3(m, name):
    a = np.asarray(m)
    if a.shape != (3, 3):
        raise ValueError(f"{name} must have shape (3,3), got {a.shape}")
    return np.asfortranarray(a, dtype=np.complex128)


def _call(name, *args):
    return _lib.call(name, *args)


# ---------------------------------------------------------------------------
# routines of c_wrapper/FLUE_c.f90
# ---------------------------------------------------------------------------
def multiplymatmat_c(left, right):
    """mm = multiplymatmat_c(left, right) (c_wrapper/FLUE_c.f90:31-36):
    MM = left . right, 3x3 complex128."""
    l, r = _mat3(left, "left"), _mat3(right, "right")
    mm = np.zeros((3, 3), dtype=np.complex128, order="F")
    _call("flue_multiplymatmat_c", _p(mm), _p(l), _p(r))
    return mm


def scalargluonprop_c(u, xi, ns=None, nt=None):
    """d = scalargluonprop_c(u, xi, [ns, nt]) (c_wrapper/FLUE_c.f90:9-16):
    the scalar gluon propagator of the position-space field U(NT,NS,NS,NS,4,3,3)
    on every lattice momentum, float64 of shape (NT,NS,NS,NS) (the reference
    declares D(NS,NS,NS,NS), which holds it only when NT = NS)."""
    a, dims = _field(u, nt=nt)
    if ns is not None and any(int(ns) != d for d in dims[1:]):
        raise ValueError(f"ns={ns} does not match the spatial extents {dims[1:]}")
    if not dims[1] == dims[2] == dims[3]:
        raise ValueError("scalargluonprop_c needs NX = NY = NZ = NS")
    return _prop.scalargluonprop(a, float(xi))


def calc_mom_space_scalard_c(u, mu_start, xi, ns=None, nt=None):
    """d = calc_mom_space_scalard_c(u, mu_start, xi, [ns, nt])
    (c_wrapper/FLUE_c.f90:18-29): the propagator on the momenta 0..N/2 of
    every axis, complex128 of shape (NT/2+1, NS/2+1, NS/2+1, NS/2+1) as the
    reference declares D(0:NT/2, 0:NS/2, 0:NS/2, 0:NS/2); mu_start 0 sums all
    four directions, 1 the spatial ones (src/gluonCalc/gluonProp.f90:165, :186)."""
    a, dims = _field(u, nt=nt)
    if ns is not None and any(int(ns) != d for d in dims[1:]):
        raise ValueError(f"ns={ns} does not match the spatial extents {dims[1:]}")
    if int(mu_start) not in (0, 1):
        raise ValueError("mu_start must be 0 or 1")
    D = _prop.scalar_gluon_prop(a, float(xi), int(mu_start))
    return np.asfortranarray(_prop.positive_octant(np.asarray(D)), dtype=np.complex128)


def q_average_c(q, d, q_slices, nq=None):
    """(dout, qout, qcount) = q_average_c(q, d, q_slices, [nq])
    (c_wrapper/FLUE_c.f90:38-48, src/gluonAna/gpManip.f90:10-49), with the
    reference's DOUT (the first D value for every bin)."""
    q = np.asarray(q, dtype=np.float64)
    n = q.size if nq is None else int(nq)
    if n < 1 or n > q.size or n > np.asarray(d).size:
        raise ValueError("nq must be in 1..len(q) and len(d)")
    return _ana.q_average(n, q, d, int(q_slices), stat="first")


def get_qhat_c(coord, shape, a=None):
    """qhat = get_qhat_c(coord, shape, [a]) (c_wrapper/FLUE_c.f90:50-57,
    src/gluonAna/momentum.f90:8-24); a defaults to 1."""
    c = np.asarray(coord, dtype=np.float64)
    s = np.asarray(shape, dtype=np.int32)
    if c.shape != (4,) or s.shape != (4,):
        raise ValueError("coord and shape must have 4 entries")
    return _ana.get_qhat(c, s, 1.0 if a is None else float(a))


def cone_cut_c(radius, q, d, d4, nt, ns, anglein, xiin, ircutin, irradiusin, nq=None):
    """(qout, dout, d4out, qcount) = cone_cut_c(radius, q, d, d4, nt, ns,
    anglein, xiin, ircutin, irradiusin, [nq]) (c_wrapper/FLUE_c.f90:59-73,
    src/gluonAna/gpManip.f90:51-163)."""
    q = np.asarray(q, dtype=np.float64)
    if q.ndim != 2 or q.shape[1] != 4:
        raise ValueError("q must have shape (NQ,4)")
    n = q.shape[0] if nq is None else int(nq)
    if n < 0 or n > q.shape[0]:
        raise ValueError("nq must be in 0..NQ")
    return _ana.cone_cut(n, int(radius), q, d, d4, int(nt), int(ns), float(anglein), float(xiin), float(ircutin),
                         float(irradiusin))


# ---------------------------------------------------------------------------
# wloops routines of the hot path (src/wloops.F90)
# ---------------------------------------------------------------------------
def _sum_np_time(name, a, dims, *ints):
    s, n, t = ctypes.c_double(), ctypes.c_int(), ctypes.c_double()
    _call(name, _p(a), *dims, *[int(v) for v in ints], ctypes.byref(s), ctypes.byref(n), ctypes.byref(t))
    return s.value, n.value, t.value


def plaquette(data, mustart, muend, nuend, nt=None, nx=None, ny=None, nz=None):
    """(sumtrp, np, time) = plaquette(data, mustart, muend, nuend)
    (src/wloops.F90:915-1017): sum of Re Tr of the plaquettes of the planes
    mu in [mustart, muend], nu in (mu, nuend]; total (1,4,4), spatial (2,4,4),
    temporal (1,1,4).  Not divided by 3 or nP; time in seconds (device)."""
    a, dims = _field(data, nt, nx, ny, nz)
    return _sum_np_time("flue_plaquette_c", a, dims, mustart, muend, nuend)


def genplaquette(data, mustart, muend, nuend, nt=None, nx=None, ny=None, nz=None):
    """(sumtrp, np, time) = genplaquette(data, mustart, muend, nuend, [nt, nx,
    ny, nz]) (src/wloops.F90:59-127): the same sum through genericPath."""
    a, dims = _field(data, nt, nx, ny, nz)
    return _sum_np_time("flue_genplaquette_c", a, dims, mustart, muend, nuend)


def polyakov(data, nt=None, nx=None, ny=None, nz=None):
    """(sumtrp, np, time) = polyakov(data) (src/wloops.F90:1019-1069): sum over
    the spatial sites of Re Tr of the ordered product of the temporal links."""
    a, dims = _field(data, nt, nx, ny, nz)
    return _sum_np_time("flue_polyakov_c", a, dims)


def genericpath(data, coordbase, path, nt=None, nx=None, ny=None, nz=None):
    """u_xd = genericpath(data, coordbase, path) (src/wloops.F90:20-57): the
    TRANSPOSED ordered product of the links along path (entries +-1..+-4)
    from the 1-based site coordbase (t, x, y, z)."""
    a, dims = _field(data, nt, nx, ny, nz)
    cb = np.ascontiguousarray(coordbase, dtype=np.int32)
    p = np.ascontiguousarray(path, dtype=np.int32).reshape(-1)
    if cb.shape != (4,):
        raise ValueError("coordbase must have 4 entries")
    out = np.zeros((3, 3), dtype=np.complex128, order="F")
    _call("flue_genericpath_c", _p(a), *dims, _p(cb), _p(p), int(p.size), _p(out))
    return out


def wmunu(data, mu, nu, nmu, nnu, nt=None, nx=None, ny=None, nz=None):
    """loopval = wmunu(data, mu, nu, nmu, nnu) (src/wloops.F90:679-791): mean
    over all sites of Re Tr of the nmu x nnu Wilson loop in plane (mu, nu)."""
    a, dims = _field(data, nt, nx, ny, nz)
    w = ctypes.c_double()
    _call("flue_wmunu_c", _p(a), *dims, int(mu), int(nu), int(nmu), int(nnu), ctypes.byref(w))
    return w.value


def wmunutau(data, tau, mu, nu, nmu, nnu, nt=None, nx=None, ny=None, nz=None):
    """loopval = wmunutau(data, tau, mu, nu, nmu, nnu) (src/wloops.F90:567-677):
    the same mean over the spatial sites of the time slice tau (1-based)."""
    a, dims = _field(data, nt, nx, ny, nz)
    w = ctypes.c_double()
    _call("flue_wmunutau_c", _p(a), *dims, int(tau), int(mu), int(nu), int(nmu), int(nnu), ctypes.byref(w))
    return w.value


def _fmunu(name, data, mu, nu, dims_kw):
    a, dims = _field(data, *dims_kw)
    out = np.zeros(dims + (3, 3), dtype=np.complex128, order="F")
    _call(name, _p(a), *dims, int(mu), int(nu), _p(out))
    return out


def cloverloopmunucoord(data, mu, nu, nt=None, nx=None, ny=None, nz=None):
    """u_xd = cloverloopmunucoord(data, mu, nu, [nt, nx, ny, nz])
    (src/wloops.F90:129-199): clover F_munu at every site, (NT,NX,NY,NZ,3,3)."""
    return _fmunu("flue_cloverloopmunucoord_c", data, mu, nu, (nt, nx, ny, nz))


def loop5munucoord(data, mu, nu, nt=None, nx=None, ny=None, nz=None):
    """u_xd = loop5munucoord(data, mu, nu, [nt, nx, ny, nz])
    (src/wloops.F90:201-432): 5-loop improved F_munu at every site."""
    return _fmunu("flue_loop5munucoord_c", data, mu, nu, (nt, nx, ny, nz))


def magnetic(data, nt=None, nx=None, ny=None, nz=None):
    """b = magnetic(data, [nt, nx, ny, nz]) (src/wloops.F90:479-544): B^2 with
    the 5-loop F of the planes (3,2), (2,4), (4,3)."""
    a, dims = _field(data, nt, nx, ny, nz)
    b = ctypes.c_double()
    _call("flue_magnetic_c", _p(a), *dims, ctypes.byref(b))
    return b.value


def magnetic_force(data, prec="c128", form="lie", nt=None, nx=None, ny=None, nz=None):
    """(b, grad) = magnetic_force(data, [prec, form]) (no reference
    counterpart): B^2 and its gradient with respect to every link, same shape
    as data; prec 'c128' (FP64), 'c64' or 'r12' (FP32 link products, FP64
    sums); form 'lie' (su(3)-projected) or 'euclid'."""
    a, dims = _field(data, nt, nx, ny, nz)
    precs = {"c128": _lib.C128, "c64": _lib.C64, "r12": _lib.R12}
    forms = {"lie": _lib.FORCE_LIE, "euclid": _lib.FORCE_EUCLID}
    if prec not in precs or form not in forms:
        raise ValueError("prec must be c128/c64/r12 and form lie/euclid")
    grad = np.zeros_like(a, order="F")
    b = ctypes.c_double()
    _call("flue_magnetic_force_c", _p(a), _lib.C128, *dims, precs[prec], forms[form], ctypes.byref(b), _p(grad))
    return b.value, grad


def uzerobar(data, g=None, nt=None, nx=None, ny=None, nz=None):
    """u0 = uzerobar(data, [g]) (README.md:17; the reference has no code):
    [u0, u0_s, u0_t] from the plaquette and the Landau-gauge mean link
    [uL, uL_s, uL_t] when the gauge transformation g(NT,NX,NY,NZ,3,3) is
    given (NaN otherwise)."""
    a, dims = _field(data, nt, nx, ny, nz)
    gp = None
    if g is not None:
        ga = np.asarray(g)
        if ga.shape != dims + (3, 3):
            raise ValueError(f"g must have shape {dims + (3, 3)}")
        ga = np.asfortranarray(ga, dtype=np.complex128)
        gp = _p(ga)
    u0 = np.zeros(6, dtype=np.float64)
    _call("flue_uzerobar_c", _p(a), *dims, gp, _p(u0))
    return u0


def fixsu3matrix(u_x):
    """fixsu3matrix(u_x) (src/gaugeIO/ILDG_bin.f90:138-151), intent(inout):
    reunitarises the 3x3 complex128 Fortran-contiguous array in place."""
    if not isinstance(u_x, np.ndarray) or u_x.dtype != np.complex128 or u_x.shape != (3, 3):
        raise ValueError("u_x must be a complex128 numpy array of shape (3,3) (intent(inout))")
    if not u_x.flags.f_contiguous:
        raise ValueError("u_x must be Fortran-contiguous (intent(inout))")
    _call("flue_fixsu3matrix_c", _p(u_x))


# FLUE_c.f90-style names of the wloops routines
plaquette_c = plaquette
genplaquette_c = genplaquette
polyakov_c = polyakov
genericpath_c = genericpath
wmunu_c = wmunu
wmunutau_c = wmunutau
cloverloopmunucoord_c = cloverloopmunucoord
loop5munucoord_c = loop5munucoord
magnetic_c = magnetic
uzerobar_c = uzerobar
fixsu3matrix_c = fixsu3matrix
