"""The wloops observables (src/wloops.F90) under FLUE.gluonCalc.

A numpy field (the reference's data(NT,NX,NY,NZ,4,3,3), from its readers or
from f2py) goes through ``flue_c``, the host-buffer tier: the call copies
the field to the GPU and returns numpy results, exactly as the f2py module
would.  A field already on the GPU -- a ``flue_gb300.GaugeField`` or a CUDA
torch tensor of that shape -- stays there (``flue_gb300.gluonCalc``, the
device tier), and matrix-valued results come back as CUDA tensors.
"""
from __future__ import annotations

import numpy as np

from FLUE.compiled import flue_c as fc


def _on_device(data) -> bool:
    from flue_gb300.field import GaugeField

    if isinstance(data, GaugeField):
        return True
    try:
        import torch

        return isinstance(data, torch.Tensor) and data.is_cuda
    except ImportError:  # pragma: no cover
        return False


def _dev():
    from flue_gb300 import gluonCalc

    return gluonCalc


def plaquette(data, mustart, muend, nuend):
    """(sumtrp, np, time) -- src/wloops.F90:915-1017"""
    if _on_device(data):
        return _dev().plaquette(data, mustart, muend, nuend)
    return fc.plaquette(data, mustart, muend, nuend)


def genplaquette(data, mustart, muend, nuend):
    """(sumtrp, np, time) -- src/wloops.F90:59-127"""
    if _on_device(data):
        return _dev().genplaquette(data, mustart, muend, nuend)
    return fc.genplaquette(data, mustart, muend, nuend)


def polyakov(data):
    """(sumtrp, np, time) -- src/wloops.F90:1019-1069"""
    if _on_device(data):
        return _dev().polyakov(data)
    return fc.polyakov(data)


def genericpath(data, coordbase, path):
    """transposed path product (3,3) -- src/wloops.F90:20-57"""
    if _on_device(data):
        return _dev().genericpath(data, coordbase, path)
    return fc.genericpath(data, coordbase, path)


def wmunu(data, mu, nu, nmu, nnu):
    """mean Re Tr of the nmu x nnu loop -- src/wloops.F90:679-791"""
    if _on_device(data):
        return _dev().wmunu(data, mu, nu, nmu, nnu)
    return fc.wmunu(data, mu, nu, nmu, nnu)


def wmunutau(data, tau, mu, nu, nmu, nnu):
    """the same on the time slice tau -- src/wloops.F90:567-677"""
    if _on_device(data):
        return _dev().wmunutau(data, tau, mu, nu, nmu, nnu)
    return fc.wmunutau(data, tau, mu, nu, nmu, nnu)


def cloverloopmunucoord(data, mu, nu):
    """clover F_munu (NT,NX,NY,NZ,3,3) -- src/wloops.F90:129-199"""
    if _on_device(data):
        return _dev().cloverloopmunucoord(data, mu, nu)
    return fc.cloverloopmunucoord(data, mu, nu)


def loop5munucoord(data, mu, nu):
    """5-loop F_munu (NT,NX,NY,NZ,3,3) -- src/wloops.F90:201-432"""
    if _on_device(data):
        return _dev().loop5munucoord(data, mu, nu)
    return fc.loop5munucoord(data, mu, nu)


def magnetic(data):
    """B^2 -- src/wloops.F90:479-544"""
    if _on_device(data):
        return _dev().magnetic(data)
    return fc.magnetic(data)


def magnetic_force(data, prec="c128", form="lie"):
    """(B^2, dB^2/dU) -- no reference counterpart"""
    if _on_device(data):
        from flue_gb300 import forces

        return forces.magnetic_force(data, form=form, prec=None if prec == "c128" else prec)
    return fc.magnetic_force(data, prec=prec, form=form)


def uzerobar(data, G=None):
    """[u0, u0_s, u0_t, uL, uL_s, uL_t] -- README.md:17 (no reference code)"""
    if _on_device(data):
        return _dev().uzerobar(data, G)
    return fc.uzerobar(data, None if G is None else np.asarray(G))
