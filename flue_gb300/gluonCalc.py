"""FLUE-compatible API for the gluonic-observable path (``FLUE.gluonCalc``).

Mirrors the reference's Python package (python/FLUE/gluonCalc) and extends
the f2py conventions of c_wrapper/FLUE_c.f90 to the routines of
src/wloops.F90: lower-case names, ``intent(in)`` arrays first, lattice
extents inferred from the array shape, ``intent(out)`` values returned (as a
tuple when there are several), 1-based directions / coordinates / path
entries, and ``ValueError`` / ``TypeError`` on bad shapes or dtypes.

``data`` is the gauge field ``data[t,x,y,z,mu,a,b]``: a numpy array, a torch
tensor (host or CUDA), or a :class:`~flue_gb300.field.GaugeField`.  Array
outputs come back as numpy arrays when ``data`` was a numpy array (f2py
style) and as CUDA tensors otherwise.  Every computation runs in the CUDA
kernels of ``libflue_gb300.so``; there is no CPU fallback.

Extra keyword ``prec`` ("c128", "c64", "r12") selects the arithmetic:
FP64 for "c128" (the reference's precision), FP32 link products with FP64
global sums for "c64" and "r12".
"""
from __future__ import annotations

import ctypes

import numpy as np
import torch

from . import _lib
from .field import GaugeField, PRECS, _ptr, _stream_handle, as_field, workspace

__all__ = [
    "multiplymatmat",
    "multiplymatdagmatdag",
    "plaquette",
    "genplaquette",
    "polyakov",
    "genericpath",
    "genericpath_all",
    "wmunu",
    "wmunutau",
    "wmunu_table",
    "cloverloopmunucoord",
    "loop5munucoord",
    "magnetic",
    "periodcoord",
    "uzerobar",
    "fixsu3matrix",
]


def _is_numpy(x) -> bool:
    return isinstance(x, np.ndarray) or (not isinstance(x, (torch.Tensor, GaugeField)) and np.ndim(x) > 0)


def _out(x: torch.Tensor, like_numpy: bool):
    if like_numpy:
        return np.asfortranarray(x.cpu().numpy())
    return x


def _scalars(t: torch.Tensor):
    return t.cpu().tolist()


class _Timer:
    """CUDA-event timer on the current stream (seconds), standing in for the
    reference's M_stopwatch wall timers (src/wloops.F90:75-76, :122-125)."""

    def __enter__(self):
        self.e0 = torch.cuda.Event(enable_timing=True)
        self.e1 = torch.cuda.Event(enable_timing=True)
        self.e0.record()
        return self

    def __exit__(self, *exc):
        self.e1.record()

    def seconds(self):
        self.e1.synchronize()
        return self.e0.elapsed_time(self.e1) * 1e-3


# ---------------------------------------------------------------------------
# SU(3) algebra (src/SU3MatrixOps.f90)
# ---------------------------------------------------------------------------
def _matmul(left, right, dagger: int):
    like_np = _is_numpy(left)
    l = torch.as_tensor(left)
    r = torch.as_tensor(right)
    if l.shape != r.shape or l.shape[-2:] != (3, 3):
        raise ValueError(f"multiplymatmat needs two (...,3,3) arrays of the same shape, got {l.shape}, {r.shape}")
    dt = torch.complex128 if (l.dtype == torch.complex128 or r.dtype == torch.complex128 or not l.is_complex()) \
        else torch.complex64
    dev = l.device if l.is_cuda else torch.device("cuda")
    batch = l.shape[:-2]
    n = int(np.prod(batch)) if len(batch) else 1
    # kernel layout: n matrices of 9 complex in Fortran order (a + 3b)
    lf = l.to(dev, dt).reshape(n, 3, 3).transpose(1, 2).contiguous()
    rf = r.to(dev, dt).reshape(n, 3, 3).transpose(1, 2).contiguous()
    of = torch.empty_like(lf)
    with torch.cuda.device(dev):
        _lib.call("flue_multiplymatmat_batch", _ptr(lf), _ptr(rf), _ptr(of), n,
                  _lib.C128 if dt == torch.complex128 else _lib.C64, dagger, _stream_handle())
    o = of.transpose(1, 2).reshape(*batch, 3, 3)
    return _out(o, like_np)


def multiplymatmat(left, right):
    """MultiplyMatMat (src/SU3MatrixOps.f90:19-37; c_wrapper/FLUE_c.f90:31-36):
    ``left @ right`` for 3x3 complex matrices, batched over leading axes."""
    return _matmul(left, right, 0)


def multiplymatdagmatdag(left, right):
    """MultiplyMatdagMatdag (src/SU3MatrixOps.f90:39-58): ``left^+ @ right^+``
    -- what the reference's code computes (its comment says (left*right)^+)."""
    return _matmul(left, right, 1)


# ---------------------------------------------------------------------------
# plaquettes, Polyakov loop (src/wloops.F90:59-127, :915-1069)
# ---------------------------------------------------------------------------
def _nplanes(mustart, muend, nuend):
    return sum(1 for mu in range(mustart, muend + 1) for nu in range(mu + 1, nuend + 1))


def plaquette(data, mustart, muend, nuend, prec=None):
    """plaquette(data, muStart, muEnd, nuEnd) -> (sumTrP, nP, time)
    (src/wloops.F90:915-1017).  sumTrP is the raw sum of Re Tr P (no 1/3);
    total = (1,4,4), spatial = (2,4,4), temporal = (1,1,4); ``time`` is the
    kernels' device time in seconds."""
    f = as_field(data, prec)
    ws = workspace(_lib.OP_PLAQUETTE, f)
    out = torch.empty(1, dtype=torch.float64, device=f.device)
    d = f.descriptor()
    with torch.cuda.device(f.device), _Timer() as tm:
        _lib.call("flue_plaquette", ctypes.byref(d), int(mustart), int(muend), int(nuend), _ptr(out), _ptr(ws),
                  ws.numel(), _stream_handle())
    s = _scalars(out)[0]
    return s, _nplanes(mustart, muend, nuend) * f.volume, tm.seconds()


def genplaquette(data, mustart, muend, nuend, prec=None):
    """genPlaquette(data,NT,NX,NY,NZ,muStart,muEnd,nuEnd) -> (sumTrP, nP, time)
    (src/wloops.F90:59-127); the extents are taken from ``data``.  Same
    observable as :func:`plaquette`."""
    return plaquette(data, mustart, muend, nuend, prec)


def polyakov(data, prec=None, return_imag=False):
    """polyakov(data) -> (sumTrP, nP, time) (src/wloops.F90:1019-1069): the
    sum over spatial sites of Re Tr of the ordered product of U_t along t.
    The reference defines the loop for NT >= 3; here every NT >= 1 gives the
    full product.  ``return_imag=True`` appends the sum of Im Tr."""
    f = as_field(data, prec)
    ws = workspace(_lib.OP_POLYAKOV, f)
    out = torch.empty(2, dtype=torch.float64, device=f.device)
    d = f.descriptor()
    with torch.cuda.device(f.device), _Timer() as tm:
        _lib.call("flue_polyakov", ctypes.byref(d), _ptr(out), _ptr(ws), ws.numel(), _stream_handle())
    re, im = _scalars(out)
    nt, nx, ny, nz = f.dims
    res = (re, nx * ny * nz, tm.seconds())
    return res + (im,) if return_imag else res


# ---------------------------------------------------------------------------
# generic path (src/wloops.F90:20-57)
# ---------------------------------------------------------------------------
def _path_array(path):
    p = np.asarray(path, dtype=np.int32).reshape(-1)
    if p.size > 256:
        raise ValueError("path longer than 256 steps")
    return np.ascontiguousarray(p)


def genericpath(data, coordbase, path, prec=None):
    """genericPath(data, coordBase, path) -> U_xd(3,3): the TRANSPOSE of the
    ordered product of links along ``path`` (entries +-1..+-4, 1-based
    directions; a negative entry steps backwards and takes the dagger of the
    forward link there) starting at the 1-based coordinate ``coordBase``."""
    like_np = _is_numpy(data) or isinstance(coordbase, (list, tuple, np.ndarray))
    f = as_field(data, prec)
    p = _path_array(path)
    cb = np.ascontiguousarray(np.asarray(coordbase, dtype=np.int32).reshape(4))
    out = torch.empty(9, dtype=f.compute_dtype, device=f.device)
    d = f.descriptor()
    with torch.cuda.device(f.device):
        _lib.call("flue_genericpath", ctypes.byref(d), cb.ctypes.data_as(ctypes.c_void_p),
                  p.ctypes.data_as(ctypes.c_void_p), int(p.size), _ptr(out), _stream_handle())
    m = out.reshape(3, 3).t()  # Fortran order (a + 3b) -> [a, b]
    return _out(m, like_np)


def genericpath_all(data, path, prec=None):
    """genericPath at every site: array (NT,NX,NY,NZ,3,3) of transposed path
    products (the batched form used by the build's API)."""
    like_np = _is_numpy(data)
    f = as_field(data, prec)
    p = _path_array(path)
    nt, nx, ny, nz = f.dims
    out = torch.empty((3, 3, nz, ny, nx, nt), dtype=f.compute_dtype, device=f.device)
    d = f.descriptor()
    with torch.cuda.device(f.device):
        _lib.call("flue_genericpath", ctypes.byref(d), None, p.ctypes.data_as(ctypes.c_void_p), int(p.size),
                  _ptr(out), _stream_handle())
    return _out(out.permute(5, 4, 3, 2, 1, 0), like_np)


# ---------------------------------------------------------------------------
# Wilson loops (src/wloops.F90:567-791)
# ---------------------------------------------------------------------------
def _wloop(f: GaugeField, tau, mu, nu, nmu, nnu, out: torch.Tensor, idx: int):
    ws = workspace(_lib.OP_WMUNU, f)
    d = f.descriptor()
    view = out[idx:idx + 1]
    _lib.call("flue_wmunu", ctypes.byref(d), int(tau), int(mu), int(nu), int(nmu), int(nnu), _ptr(view), _ptr(ws),
              ws.numel(), _stream_handle())


def wmunu(data, mu, nu, nmu, nnu, prec=None):
    """wmunu(data, mu, nu, nMu, nNu) -> loopVal (src/wloops.F90:679-791): the
    mean over all sites of Re Tr of the nMu x nNu loop in plane (mu,nu)."""
    f = as_field(data, prec)
    out = torch.empty(1, dtype=torch.float64, device=f.device)
    with torch.cuda.device(f.device):
        _wloop(f, 0, mu, nu, nmu, nnu, out, 0)
    return _scalars(out)[0]


def wmunutau(data, tau, mu, nu, nmu, nnu, prec=None):
    """wmunutau(data, tau, mu, nu, nMu, nNu) -> loopVal (src/wloops.F90:567-677):
    the mean over the spatial sites of the slice t = tau (1-based)."""
    f = as_field(data, prec)
    if not 1 <= int(tau) <= f.nt:
        raise ValueError("tau must be in 1..NT")
    out = torch.empty(1, dtype=torch.float64, device=f.device)
    with torch.cuda.device(f.device):
        _wloop(f, tau, mu, nu, nmu, nnu, out, 0)
    return _scalars(out)[0]


def wmunu_table(data, mu, nu, rmax, tmax, prec=None):
    """All wmunu(data, mu, nu, R, T) for R in 1..rmax, T in 1..tmax as an
    (rmax, tmax) array, from lines built once per site (flue_wmunu_table)."""
    f = as_field(data, prec)
    L = _lib.load()
    nt, nx, ny, nz = f.dims
    nb = L.flue_wmunu_table_bytes(nt, nx, ny, nz, PRECS[f.prec], int(rmax), int(tmax))
    ws = torch.empty(max(nb, 256), dtype=torch.uint8, device=f.device)
    out = torch.empty(rmax * tmax, dtype=torch.float64, device=f.device)
    d = f.descriptor()
    with torch.cuda.device(f.device):
        _lib.call("flue_wmunu_table", ctypes.byref(d), int(mu), int(nu), int(rmax), int(tmax), _ptr(out), _ptr(ws),
                  ws.numel(), _stream_handle())
    return np.asarray(_scalars(out)).reshape(rmax, tmax)


# ---------------------------------------------------------------------------
# F_munu and B^2 (src/wloops.F90:129-544)
# ---------------------------------------------------------------------------
def _fmunu(data, kind, mu, nu, prec):
    like_np = _is_numpy(data)
    f = as_field(data, prec)
    nt, nx, ny, nz = f.dims
    ws = workspace(_lib.OP_FMUNU, f)
    out = torch.empty((3, 3, nz, ny, nx, nt), dtype=f.compute_dtype, device=f.device)
    d = f.descriptor()
    with torch.cuda.device(f.device):
        _lib.call("flue_fmunu", ctypes.byref(d), kind, int(mu), int(nu), _ptr(out), _ptr(ws), ws.numel(),
                  _stream_handle())
    return _out(out.permute(5, 4, 3, 2, 1, 0), like_np)


def cloverloopmunucoord(data, mu, nu, prec=None):
    """cloverLoopMuNuCoord(data,NT,NX,NY,NZ,mu,nu) -> (NT,NX,NY,NZ,3,3)
    (src/wloops.F90:129-199): clover F_munu, anti-Hermitian (not traceless)
    projection times 1/4."""
    return _fmunu(data, _lib.FMUNU_CLOVER, mu, nu, prec)


def loop5munucoord(data, mu, nu, prec=None):
    """Loop5MuNuCoord(data,NT,NX,NY,NZ,mu,nu) -> (NT,NX,NY,NZ,3,3)
    (src/wloops.F90:201-432): 5-loop improved F_munu (hep-lat/0203008)."""
    return _fmunu(data, _lib.FMUNU_LOOP5, mu, nu, prec)


def magnetic(data, prec=None):
    """magnetic(data,NT,NX,NY,NZ) -> B (src/wloops.F90:479-544):
    B^2 = (1/V) sum_x sum_i -Re Tr(F_i F_i) with the 5-loop F of the
    planes (3,2), (2,4), (4,3)."""
    f = as_field(data, prec)
    ws = workspace(_lib.OP_MAGNETIC, f)
    out = torch.empty(1, dtype=torch.float64, device=f.device)
    d = f.descriptor()
    with torch.cuda.device(f.device):
        _lib.call("flue_magnetic", ctypes.byref(d), _ptr(out), _ptr(ws), ws.numel(), _stream_handle())
    return _scalars(out)[0]


# ---------------------------------------------------------------------------
# helpers of the reference interface
# ---------------------------------------------------------------------------
def periodcoord(coord, datashape):
    """periodCoord(coord, dataShape) (src/wloops.F90:546-565): a coordinate
    component above its extent becomes 1, a zero becomes the extent (only
    +-1 steps are handled, like the reference).  Integer bookkeeping for
    host callers; the kernels wrap coordinates themselves."""
    c = [int(v) for v in coord]
    for k in range(4):
        if c[k] > int(datashape[k]):
            c[k] = 1
        elif c[k] == 0:
            c[k] = int(datashape[k])
    return np.asarray(c, dtype=np.int32)


def uzerobar(data, G=None, prec=None):
    """uzerobar (README.md:17; the reference ships no code for it).
    Returns a length-6 array: [u0, u0_s, u0_t] from the plaquette,
    u0 = (<Re Tr P>/3)^(1/4) over all planes, u0_s from the spatial planes,
    u0_t = (<Re Tr P_st>/3)^(1/2) / u0_s; then the Landau-gauge mean link
    [uL, uL_s, uL_t] = <Re Tr(G(x) U_mu(x) G(x+mu)^+)>/3 over all, spatial and
    temporal links when the gauge transformation G (NT,NX,NY,NZ,3,3) is
    given (NaN otherwise).  Sums and roots in FP64."""
    f = as_field(data, prec)
    V = float(f.volume)
    res = np.full(6, np.nan)
    out = torch.empty(7, dtype=torch.float64, device=f.device)
    d = f.descriptor()
    ws = workspace(_lib.OP_PLAQUETTE, f)
    with torch.cuda.device(f.device):
        for k, (a, b, c) in enumerate(((1, 4, 4), (2, 4, 4), (1, 1, 4))):
            _lib.call("flue_plaquette", ctypes.byref(d), a, b, c, _ptr(out[k:k + 1]), _ptr(ws), ws.numel(),
                      _stream_handle())
        if G is not None:
            g = torch.as_tensor(G)
            if tuple(g.shape) != tuple(f.dims) + (3, 3):
                raise ValueError("G must have shape (NT,NX,NY,NZ,3,3)")
            gd = g.to(f.device).permute(5, 4, 3, 2, 1, 0).contiguous()
            if gd.dtype not in (torch.complex128, torch.complex64):
                raise TypeError("G must be complex128 or complex64")
            ws2 = workspace(_lib.OP_MEANLINK, f)
            _lib.call("flue_meanlink", ctypes.byref(d), _ptr(gd),
                      _lib.C128 if gd.dtype == torch.complex128 else _lib.C64, _ptr(out[3:7]), _ptr(ws2),
                      ws2.numel(), _stream_handle())
    s = _scalars(out)
    p = np.array([s[0] / (6 * V) / 3, s[1] / (3 * V) / 3, s[2] / (3 * V) / 3])
    with np.errstate(invalid="ignore"):  # a negative mean plaquette has no real root: NaN
        res[0] = np.power(p[0], 0.25)
        res[1] = np.power(p[1], 0.25)
        res[2] = np.sqrt(p[2]) / res[1]
    if G is not None:
        res[3] = (s[3] + s[4] + s[5] + s[6]) / (4 * V) / 3
        res[4] = (s[4] + s[5] + s[6]) / (3 * V) / 3
        res[5] = s[3] / V / 3
    return res


def fixsu3matrix(u):
    """FixSU3Matrix (src/gaugeIO/ILDG_bin.f90:138-151) of one 3x3 matrix or a
    batch (...,3,3): Gram-Schmidt on the rows, third row conj(r1 x r2)."""
    like_np = _is_numpy(u)
    m = torch.as_tensor(u)
    if m.shape[-2:] != (3, 3):
        raise ValueError("fixsu3matrix needs (...,3,3) matrices")
    batch = m.shape[:-2]
    n = int(np.prod(batch)) if len(batch) else 1
    dev = m.device if m.is_cuda else torch.device("cuda")
    src = m.to(dev, torch.complex128).reshape(n, 3, 3).contiguous()
    # treat the n matrices as a 1-direction-repeated field of extent (n,1,1,1)
    dst = torch.empty((3, 3, 4, 1, 1, 1, n), dtype=torch.complex128, device=dev)
    strides = (ctypes.c_int64 * 7)(9, 0, 0, 0, 0, 3, 1)
    with torch.cuda.device(dev):
        _lib.call("flue_pack_field", _ptr(src), _lib.C128, strides, n, 1, 1, 1, _ptr(dst), _lib.C128, 1,
                  _stream_handle())
    o = dst[:, :, 0, 0, 0, 0, :].permute(2, 1, 0).reshape(*batch, 3, 3)
    return _out(o, like_np)
