"""Jackknife statistics over configurations (src/jack.f90), used by the
reference's magnetic workflow to turn per-configuration B^2 and plaquettes
into means with errors (app/magnetic.f90:143-160).  Host-side numpy: the
work is O(number of configurations)."""
from __future__ import annotations

import numpy as np


def complement(data, drop=()):
    """Complement0..3 (src/jack.f90:18-46).

    ``complement(data)`` -> the mean (Complement0);
    ``complement(data, ('all',))`` -> the first-order jackknife means with
    each configuration left out (Complement1);
    ``complement(data, (i,))`` / ``(i, j)`` -> second / third order sets with
    configuration(s) i (and j, 0-based) also left out (Complement2/3)."""
    d = np.asarray(data, dtype=np.float64)
    n = d.size
    if not drop:
        return float(d.sum() / n)
    if drop == ("all",):
        return (d.sum() - d) / (n - 1)
    extra = float(sum(d[i] for i in drop))
    return (d.sum() - extra - d) / (n - 1 - len(drop))


def jackknife_wp(c):
    """JackKnife_wp (src/jack.f90:48-59): c[0] is the full-sample mean,
    c[1:] the first-order jackknife means.  Returns (err, bias)."""
    c = np.asarray(c, dtype=np.float64)
    avg = c[1:].sum() / (c.size - 1)
    err = np.sqrt(np.sum((c[1:] - avg) ** 2) * (c.size - 2) / (c.size - 1))
    return float(err), float(c[0] - avg)


def mean_and_error(data):
    """The magnetic app's summary of one observable (app/magnetic.f90:143-157):
    full mean and first-order jackknife error."""
    c = np.concatenate([[complement(data)], complement(data, ("all",))])
    err, _ = jackknife_wp(c)
    return c[0], err
