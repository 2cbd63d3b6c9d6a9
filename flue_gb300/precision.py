"""Per-observable error of the FP32 forms (complex64 full 18-real and
reconstruct-12) against the FP64 kernels on the same field.

FP32 runs the link products in single precision and keeps every global sum,
the u0 roots and the reunitarisation in FP64; this module measures what that
costs for each observable: plaquettes, Polyakov loop, 5-loop F_munu
components, B^2, u0 and the B^2 gradient.
"""
from __future__ import annotations

from typing import Dict, Sequence

import numpy as np
import torch

from . import forces, gluonCalc as G
from .field import GaugeField


def _rel(a, b):
    return float(abs(a - b) / abs(b)) if b != 0 else float(abs(a - b))


def observables(f: GaugeField, planes=((3, 2), (1, 4))) -> Dict[str, object]:
    out = {}
    for name, r in (("plaq_all", (1, 4, 4)), ("plaq_spatial", (2, 4, 4)), ("plaq_temporal", (1, 1, 4))):
        s, n, _ = G.plaquette(f, *r)
        out[name] = s / n / 3.0
    s, n, _, im = G.polyakov(f, return_imag=True)
    out["polyakov"] = complex(s, im) / n / 3.0
    for mu, nu in planes:
        out[f"F{mu}{nu}"] = G.loop5munucoord(f, mu, nu).to(torch.complex128)
    b2, g = forces.magnetic_force(f)
    out["b2"] = b2
    out["grad_b2"] = g.to(torch.complex128)
    out["u0"] = G.uzerobar(f)[:3]
    return out


def precision_report(field: GaugeField, precs: Sequence[str] = ("c64", "r12")) -> Dict[str, Dict[str, float]]:
    """Errors of each FP32 form against the FP64 evaluation of ``field``
    (which must be a c128 field): relative error for scalars, relative L2 and
    max-abs / max-abs-of-reference for matrix fields."""
    if field.prec != "c128":
        raise ValueError("precision_report needs the FP64 (c128) field as the reference")
    ref = observables(field)
    rep = {}
    for p in precs:
        cur = observables(GaugeField.from_array(field, prec=p))
        r = {}
        for k, v in ref.items():
            w = cur[k]
            if isinstance(v, torch.Tensor):
                d = (w - v)
                r[k + "_rel_l2"] = float(torch.linalg.vector_norm(d.flatten()) / torch.linalg.vector_norm(v.flatten()))
                r[k + "_max_rel"] = float(d.abs().max() / v.abs().max())
            elif isinstance(v, np.ndarray):
                r[k] = float(np.max(np.abs(w - v) / np.abs(v)))
            elif isinstance(v, complex):
                r[k] = float(abs(w - v) / abs(v))
            else:
                r[k] = _rel(w, v)
        rep[p] = r
    rep["fp64_values"] = {k: (v if isinstance(v, float) else (str(v) if isinstance(v, complex) else None))
                          for k, v in ref.items() if not isinstance(v, torch.Tensor)}
    return rep
