"""Scalar gluon propagator and gauge transformation on the GPU.

The reference works towards a gluon propagator in
``src/gluonCalc/gluonProp.f90`` (``scalarGluonProp``,
``calc_mom_space_scalarD``) but its routines are unfinished; what is
computed here is the definition they cite, hep-lat/9803105:

    A_mu(x)   = [U_mu(x) - U_mu(x)^+] / (2i) - Tr/3,   A^a = Tr(A lambda^a)
    A^a_mu(q) = sum_x exp(-i q.x) A^a_mu(x),             q_mu = 2 pi n_mu / N_mu
    D(q)      = sum_{mu >= mu_start} w_mu sum_a |A^a_mu(q)|^2 / (8 n(q) V)
              = 2 / ((Nc^2-1) n(q) V) sum_mu w_mu Tr[A_mu(q) A_mu(-q)]

with w_t = xi^2 (anisotropy), w_i = 1, n(0) = 4, n(q != 0) = 3.  The field
must be in Landau gauge: apply the gauge transformation that
``gaugeIO.read_gauge_transformation_cola`` reads with ``gauge_transform``.
"""
from __future__ import annotations

import ctypes

import numpy as np
import torch

from . import _lib
from .field import GaugeField, _ptr, _stream_handle, as_field, workspace
from .gluonCalc import _is_numpy, _out


def scalar_gluon_prop(data, xi: float = 1.0, mu_start: int = 0, prec=None):
    """D(q) on every lattice momentum, shape (NT,NX,NY,NZ), FP64; index n_mu
    = 0..N_mu-1 with n_mu > N_mu/2 the negative momenta.  ``mu_start`` = 0
    sums all four directions, 1 the spatial ones (gluonProp.f90:165, 186).
    numpy in -> numpy out; a GaugeField or tensor gives a device tensor."""
    if mu_start not in (0, 1):
        raise ValueError("mu_start must be 0 or 1")
    like_np = _is_numpy(data)
    f = as_field(data, prec)
    nt, nx, ny, nz = f.dims
    ws = workspace(_lib.OP_GLUON_PROP, f)
    out = torch.empty((nz, ny, nx, nt), dtype=torch.float64, device=f.device)
    d = f.descriptor()
    with torch.cuda.device(f.device):
        _lib.call("flue_gluon_propagator", ctypes.byref(d), float(xi), int(mu_start), _ptr(out), _ptr(ws),
                  ws.numel(), _stream_handle())
    return _out(out.permute(3, 2, 1, 0), like_np)


def scalargluonprop(U, xi: float = 1.0):
    """scalarGluonProp_c(NS, NT, U, xi) -> D (c_wrapper/FLUE_c.f90:9-16)
    through the host-buffer C entry: U a complex128 (NT,NS,NS,NS,4,3,3) numpy
    array, D a float64 (NT,NS,NS,NS) numpy array (all four directions)."""
    a = np.asfortranarray(U, dtype=np.complex128)
    nt, ns = a.shape[0], a.shape[1]
    if a.shape != (nt, ns, ns, ns, 4, 3, 3):
        raise ValueError("U must have shape (NT,NS,NS,NS,4,3,3)")
    D = np.zeros((nt, ns, ns, ns), dtype=np.float64, order="F")
    _lib.call("flue_scalargluonprop_c", ns, nt, a.ctypes.data_as(ctypes.c_void_p), float(xi),
              D.ctypes.data_as(ctypes.c_void_p))
    return D


def positive_octant(D):
    """The momenta 0..N_mu/2 of every axis, the output range of
    calc_mom_space_scalarD (D(0:NT/2, 0:NS/2, 0:NS/2, 0:NS/2),
    gluonProp.f90:125)."""
    nt, nx, ny, nz = D.shape
    return D[: nt // 2 + 1, : nx // 2 + 1, : ny // 2 + 1, : nz // 2 + 1]


def gauge_transform(field: GaugeField, G) -> GaugeField:
    """U_mu(x) <- G(x) U_mu(x) G(x+mu)^+ in place on a device field; G of
    shape (NT,NX,NY,NZ,3,3), complex128 or complex64, SU(3)."""
    if not isinstance(field, GaugeField):
        raise TypeError("gauge_transform works in place on a GaugeField")
    g = torch.as_tensor(G)
    if tuple(g.shape) != tuple(field.dims) + (3, 3):
        raise ValueError("G must have shape (NT,NX,NY,NZ,3,3)")
    if g.dtype not in (torch.complex128, torch.complex64):
        raise TypeError("G must be complex128 or complex64")
    gd = g.to(field.device).permute(5, 4, 3, 2, 1, 0).contiguous()
    d = field.descriptor()
    with torch.cuda.device(field.device):
        _lib.call("flue_gauge_transform", ctypes.byref(d), _ptr(gd),
                  _lib.C128 if gd.dtype == torch.complex128 else _lib.C64, _stream_handle())
    return field
