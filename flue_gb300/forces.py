"""Gradients of the gluonic observables (no reference counterpart).

For an observable O and a link U = U_mu(x), N denotes the matrix with
dO = Re Tr(dU N) for every variation dU.  Two forms are returned:

* ``form="lie"``: the su(3)-projected Lie derivative
  G = sum_a T^a d/dh O(e^{h T^a} U)|_{h=0} = -1/2 TA(U N), T^a = i lambda^a/2,
  so that the directional derivative along X in su(3) is D_X O = -2 Re Tr(X G).
* ``form="euclid"``: dO/d(Re U) + i dO/d(Im U) = N^+, the convention of
  ``torch.autograd`` for complex inputs.

Outputs have the field's shape (NT,NX,NY,NZ,4,3,3): complex128 for FP64
fields, complex64 for FP32 ones.  The kernels recompute leaves from the
links (only F = dE/dQ is kept between the forward and backward sweeps).
"""
from __future__ import annotations

import ctypes

import numpy as np
import torch

from . import _lib
from .field import GaugeField, _ptr, _stream_handle, as_field, workspace

B2_PLANES = ((3, 2), (2, 4), (4, 3))
ALL_PLANES = ((1, 2), (1, 3), (1, 4), (2, 3), (2, 4), (3, 4))
_FORMS = {"lie": _lib.FORCE_LIE, "euclid": _lib.FORCE_EUCLID}


def _alloc_force(f: GaugeField):
    nt, nx, ny, nz = f.dims
    return torch.empty((3, 3, 4, nz, ny, nx, nt), dtype=f.compute_dtype, device=f.device)


def _as_view(t: torch.Tensor) -> torch.Tensor:
    return t.permute(6, 5, 4, 3, 2, 1, 0)


def magnetic_force(data, form="lie", prec=None, with_force=True):
    """B^2 (magnetic, src/wloops.F90:479-544) and its gradient."""
    f = as_field(data, prec)
    ws = workspace(_lib.OP_MAGNETIC_FORCE, f)
    out = torch.empty(1, dtype=torch.float64, device=f.device)
    g = _alloc_force(f) if with_force else None
    d = f.descriptor()
    with torch.cuda.device(f.device):
        _lib.call("flue_magnetic_force", ctypes.byref(d), _ptr(out), _ptr(g) if g is not None else None,
                  _FORMS[form], _ptr(ws), ws.numel(), _stream_handle())
    return out.item(), (_as_view(g) if g is not None else None)


def loop5_energy_force(data, planes=ALL_PLANES, form="lie", prec=None):
    """E = -1/V sum_x sum_planes Re Tr(F F) with the 5-loop F of the listed
    1-based (mu,nu) planes, and its gradient."""
    f = as_field(data, prec)
    p = np.ascontiguousarray(np.asarray(planes, dtype=np.int32).reshape(-1))
    ws = workspace(_lib.OP_ENERGY_FORCE, f)
    out = torch.empty(1, dtype=torch.float64, device=f.device)
    g = _alloc_force(f)
    d = f.descriptor()
    with torch.cuda.device(f.device):
        _lib.call("flue_loop5_energy_force", ctypes.byref(d), p.ctypes.data_as(ctypes.c_void_p), len(planes),
                  _ptr(out), _ptr(g), _FORMS[form], _ptr(ws), ws.numel(), _stream_handle())
    return out.item(), _as_view(g)


def plaquette_force(data, form="lie", prec=None):
    """S = sum_{x,mu<nu} Re Tr P_munu(x) (the raw plaquette sum of
    plaquette(data,1,4,4)) and its gradient (the Wilson staple force)."""
    f = as_field(data, prec)
    ws = workspace(_lib.OP_PLAQUETTE_FORCE, f)
    out = torch.empty(1, dtype=torch.float64, device=f.device)
    g = _alloc_force(f)
    d = f.descriptor()
    with torch.cuda.device(f.device):
        _lib.call("flue_plaquette_force", ctypes.byref(d), _ptr(out), _ptr(g), _FORMS[form], _ptr(ws), ws.numel(),
                  _stream_handle())
    return out.item(), _as_view(g)


# ---------------------------------------------------------------------------
# torch.autograd front ends
# ---------------------------------------------------------------------------
class _EnergyFn(torch.autograd.Function):
    @staticmethod
    def forward(ctx, U, kind, planes):
        ctx.kind, ctx.planes = kind, planes
        ctx.save_for_backward(U)
        if kind == "b2":
            e, _ = magnetic_force(U.detach(), with_force=False)
        elif kind == "plaq":
            e, _ = plaquette_force(U.detach())
        else:
            e, _ = loop5_energy_force(U.detach(), planes)
        return torch.tensor(e, dtype=torch.float64, device=U.device)

    @staticmethod
    def backward(ctx, gout):
        (U,) = ctx.saved_tensors
        if ctx.kind == "b2":
            _, g = magnetic_force(U.detach(), form="euclid")
        elif ctx.kind == "plaq":
            _, g = plaquette_force(U.detach(), form="euclid")
        else:
            _, g = loop5_energy_force(U.detach(), ctx.planes, form="euclid")
        return g.to(U.dtype) * gout.to(g.real.dtype), None, None


def magnetic_autograd(U: torch.Tensor) -> torch.Tensor:
    """B^2 of a complex CUDA tensor U[t,x,y,z,mu,a,b] as a differentiable
    torch scalar (backward = the hand-written gradient kernels)."""
    return _EnergyFn.apply(U, "b2", None)


def loop5_energy_autograd(U: torch.Tensor, planes=ALL_PLANES) -> torch.Tensor:
    return _EnergyFn.apply(U, "e", tuple(planes))


def plaquette_action_autograd(U: torch.Tensor) -> torch.Tensor:
    return _EnergyFn.apply(U, "plaq", None)
