"""Wilson flow (Luescher, JHEP 08 (2010) 071) driven by the hand-written
plaquette-action gradient kernel, with B^2 measured along the way.

The RK3 step runs entirely on the GPU (``flue_wflow_step``); the flow time
advances by ``eps`` per step.  No reference counterpart.
"""
from __future__ import annotations

import ctypes
import os

import torch

from . import _lib, gluonCalc
from .field import GaugeField, _ptr, _stream_handle, as_field, workspace


def wflow_step(field: GaugeField, eps: float) -> GaugeField:
    """One RK3 step in place (c128 or c64 field)."""
    ws = workspace(_lib.OP_WFLOW, field)
    d = field.descriptor()
    with torch.cuda.device(field.device):
        _lib.call("flue_wflow_step", ctypes.byref(d), float(eps), _ptr(ws), ws.numel(), _stream_handle())
    return field


def wilson_flow(data, eps: float = 0.01, tmax: float = 2.0, measure_every: float = 0.1, prec=None,
                observables=("b2", "plaq"), checkpoint=None):
    """Flow ``data`` to t = tmax with step eps; every ``measure_every`` in
    flow time (and at t = 0) record t, B^2 and the mean plaquette
    <Re Tr P>/3.  Returns (flowed GaugeField, list of dict records).

    ``checkpoint``: a file path.  After every measurement the step count,
    the records and the links are saved there (torch.save, written to a
    temporary name and renamed, so an interrupted save leaves the previous
    checkpoint); a call whose checkpoint file exists, for the same lattice,
    precision and eps, continues from it instead of from ``data``.  The
    continued flow is bitwise the uninterrupted one."""
    f = as_field(data, prec)
    if f.prec == "r12":
        raise ValueError("the Wilson flow updates links in place; use a c128 or c64 field")
    f = f.clone()  # never flow the caller's links in place
    nsteps = int(round(tmax / eps))
    every = max(1, int(round(measure_every / eps)))
    recs = []
    start = 1
    if checkpoint is not None and os.path.exists(checkpoint):
        ck = torch.load(checkpoint, map_location="cpu", weights_only=False)
        if tuple(ck["dims"]) != tuple(f.dims) or ck["prec"] != f.prec or ck["eps"] != eps:
            raise ValueError("checkpoint %s is for another lattice, precision or step" % checkpoint)
        f.storage.copy_(ck["links"].to(f.device))
        recs = list(ck["recs"])
        start = ck["step"] + 1

    def measure(step):
        r = {"t": step * eps}
        if "b2" in observables:
            r["b2"] = gluonCalc.magnetic(f)
        if "plaq" in observables:
            s, n, _ = gluonCalc.plaquette(f, 1, 4, 4)
            r["plaq"] = s / n / 3.0
        recs.append(r)
        if checkpoint is not None:
            tmp = checkpoint + ".tmp"
            torch.save({"dims": f.dims, "prec": f.prec, "eps": eps, "step": step, "recs": recs,
                        "links": f.storage.detach().cpu()}, tmp)
            os.replace(tmp, checkpoint)

    if start == 1:
        measure(0)
    for k in range(start, nsteps + 1):
        wflow_step(f, eps)
        if k % every == 0:
            measure(k)
    return f, recs
