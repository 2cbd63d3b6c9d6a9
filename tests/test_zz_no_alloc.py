"""flue_plaquette_noalloc, the plaquette entry point that allocates nothing.

It exists for callers that manage all device memory themselves and cannot
let a library allocate (for instance a simulation that measures the
plaquette inside its update loop while its own pool holds the GPU memory).
Here it is called through the C ABI and compared with flue_plaquette (the
entry point that takes a workspace) on two calls in a row, with a different
plane range and lattice size on the second call, so that scratch contents
left by the first call cannot leak into the second.  The test's own field
and output buffers are allocated by torch; the entry point allocates none.
This file is collected last so that a run stopping at its first failure has
already run every other test.
"""
import ctypes

import pytest
import torch

from flue_gb300 import _lib, generate
from flue_gb300.field import GaugeField, workspace

pytestmark = pytest.mark.gpu

TOL = 1e-12  # FP64 relative, the tolerance of the other plaquette parity tests


def _with_workspace(L, f, rng):
    out = torch.zeros(1, dtype=torch.float64, device="cuda")
    ws = workspace(_lib.OP_PLAQUETTE, f)
    d = f.descriptor()
    rc = L.flue_plaquette(ctypes.byref(d), rng[0], rng[1], rng[2], ctypes.c_void_p(out.data_ptr()),
                          ctypes.c_void_p(ws.data_ptr()), ws.numel(),
                          ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
    assert rc == 0
    return out.item()


def _no_alloc(L, f, rng):
    out = torch.full((1,), float("nan"), dtype=torch.float64, device="cuda")
    d = f.descriptor()
    rc = L.flue_plaquette_noalloc(ctypes.byref(d), rng[0], rng[1], rng[2], ctypes.c_void_p(out.data_ptr()),
                                  ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
    assert rc == 0, L.flue_last_error_detail()
    return out.item()


def test_noalloc_plaquette_matches_workspace_entry_twice():
    L = _lib.load()
    f1 = generate.random_field((8, 8, 8, 8), 0.3, 41, device="cuda")
    f2 = GaugeField.from_array(generate.random_field((6, 4, 5, 3), 0.5, 42), prec="c64")
    calls = [(f1, (1, 4, 4)), (f2, (2, 4, 4))]
    for f, rng in calls:
        ref = _with_workspace(L, f, rng)
        got = _no_alloc(L, f, rng)
        assert abs(got - ref) <= TOL * abs(ref), (got, ref)


def test_noalloc_rejects_bad_arguments():
    L = _lib.load()
    f = generate.random_field((4, 4, 4, 4), 0.3, 43, device="cuda")
    d = f.descriptor()
    out = torch.zeros(1, dtype=torch.float64, device="cuda")
    assert L.flue_plaquette_noalloc(ctypes.byref(d), 0, 4, 4, ctypes.c_void_p(out.data_ptr()), None) == _lib.FLUE_ERR_ARG
    assert L.flue_plaquette_noalloc(ctypes.byref(d), 1, 4, 4, None, None) == _lib.FLUE_ERR_ARG
