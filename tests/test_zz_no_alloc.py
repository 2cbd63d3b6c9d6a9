"""flue_plaquette_noalloc, the plaquette entry point that allocates nothing.

It exists for callers that manage all device memory themselves and cannot
let a library allocate (for instance a simulation that measures the
plaquette inside its update loop while its own pool holds the GPU memory).
Here it is called through the C ABI and compared with flue_plaquette (the
entry point that takes a workspace: the same kernel and grid, so the sums
must be bitwise equal) and with the oracle, on calls in a row over the three
field precisions, with a different plane range and lattice size on each
call, so that scratch contents left by one call cannot leak into the next.
The test's own field and output buffers are allocated by torch; the entry
point allocates none.  Argument rejections return before anything touches
the GPU, so they are checked on the CPU too.  This file is collected last so
that a run stopping at its first failure has already run every other test.
"""
import ctypes

import pytest

from flue_gb300 import _lib

TOL_FP64 = 1e-12  # FP64 relative, the tolerance of the other plaquette parity tests
TOL_FP32 = 3e-6   # FP32 relative, as for the c64 / r12 plaquettes of the parity tests


def _stream():
    import torch

    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)


def _with_workspace(L, f, rng):
    import torch

    from flue_gb300.field import workspace

    out = torch.zeros(1, dtype=torch.float64, device="cuda")
    ws = workspace(_lib.OP_PLAQUETTE, f)
    d = f.descriptor()
    rc = L.flue_plaquette(ctypes.byref(d), rng[0], rng[1], rng[2], ctypes.c_void_p(out.data_ptr()),
                          ctypes.c_void_p(ws.data_ptr()), ws.numel(), _stream())
    assert rc == 0
    return out.item()


def _no_alloc(L, f, rng):
    import torch

    out = torch.full((1,), float("nan"), dtype=torch.float64, device="cuda")
    d = f.descriptor()
    rc = L.flue_plaquette_noalloc(ctypes.byref(d), rng[0], rng[1], rng[2], ctypes.c_void_p(out.data_ptr()), _stream())
    assert rc == 0, L.flue_last_error_detail()
    return out.item()


@pytest.mark.gpu
def test_noalloc_plaquette_matches_workspace_entry_and_oracle():
    import oracle
    from flue_gb300 import generate
    from flue_gb300.field import GaugeField

    L = _lib.load()
    calls = [
        ((8, 8, 8, 8), 0.3, 41, "c128", (1, 4, 4)),
        ((6, 4, 5, 3), 0.5, 42, "c64", (2, 4, 4)),
        ((5, 6, 4, 4), 0.4, 43, "r12", (1, 1, 4)),
        ((8, 8, 8, 8), 0.3, 41, "c128", (1, 4, 4)),  # the first call again, after the others
    ]
    for dims, eps, seed, prec, rng in calls:
        host = generate.random_field(dims, eps, seed)
        f = GaugeField.from_array(host, prec=prec, device="cuda")
        ref = _with_workspace(L, f, rng)
        got = _no_alloc(L, f, rng)
        assert got == ref, (prec, got, ref)
        want, _ = oracle.plaquette(host, *rng)
        tol = TOL_FP64 if prec == "c128" else TOL_FP32
        assert abs(got - want) <= tol * abs(want), (prec, got, want)


def test_noalloc_rejects_bad_arguments_before_any_launch():
    # Every case below is refused by the host-side checks, so no kernel runs
    # and no GPU is needed; the links pointers are never dereferenced.
    L = _lib.load()
    out = ctypes.c_double()
    good = _lib.FlueField(4096, 4, 4, 4, 4, _lib.C128)
    assert L.flue_plaquette_noalloc(ctypes.byref(good), 0, 4, 4, ctypes.byref(out), None) == _lib.FLUE_ERR_ARG
    assert L.flue_plaquette_noalloc(ctypes.byref(good), 1, 4, 4, None, None) == _lib.FLUE_ERR_ARG
    assert L.flue_plaquette_noalloc(None, 1, 4, 4, ctypes.byref(out), None) == _lib.FLUE_ERR_ARG
    null_links = _lib.FlueField(None, 4, 4, 4, 4, _lib.C128)
    assert L.flue_plaquette_noalloc(ctypes.byref(null_links), 1, 4, 4, ctypes.byref(out), None) == _lib.FLUE_ERR_ARG
    bad_prec = _lib.FlueField(4096, 4, 4, 4, 4, 9)
    assert L.flue_plaquette_noalloc(ctypes.byref(bad_prec), 1, 4, 4, ctypes.byref(out), None) == _lib.FLUE_ERR_DTYPE
    zero = _lib.FlueField(4096, 4, 0, 4, 4, _lib.C128)
    assert L.flue_plaquette_noalloc(ctypes.byref(zero), 1, 4, 4, ctypes.byref(out), None) == _lib.FLUE_ERR_SHAPE
    # links off their element alignment: 8 bytes for C128 and R12, 4 for C64
    for prec, off in ((_lib.C128, 8), (_lib.R12, 8), (_lib.C64, 4)):
        mis = _lib.FlueField(4096 + off, 4, 4, 4, 4, prec)
        rc = L.flue_plaquette_noalloc(ctypes.byref(mis), 1, 4, 4, ctypes.byref(out), None)
        assert rc == _lib.FLUE_ERR_LAYOUT, (prec, rc, L.flue_last_error_detail())
    # the workspace entry point refuses the same misaligned pointer
    mis = _lib.FlueField(4096 + 8, 4, 4, 4, 4, _lib.C128)
    assert L.flue_plaquette(ctypes.byref(mis), 1, 4, 4, ctypes.byref(out), None, 0, None) == _lib.FLUE_ERR_LAYOUT
