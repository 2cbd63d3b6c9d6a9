"""GPU gradients: against the oracle's brute-force reverse mode and analytic
staple force (FP64 to 1e-11), against central finite differences along random
su(3) directions (FP64, h = 1e-4), the Euclidean / Lie form relation, the
torch.autograd front end, and the FP32 error bound."""
import numpy as np
import pytest
import torch

import oracle
from flue_gb300 import forces, generate, gluonCalc as G
from flue_gb300.field import GaugeField
from tests import np_flue

pytestmark = pytest.mark.gpu


def _np(t):
    return t.detach().cpu().numpy() if isinstance(t, torch.Tensor) else t


def _lie_pair(g, x):
    return float(-2.0 * np.einsum("...ij,...ji->...", x, g).real.sum())


def _perturb(U, X, h):
    return np.asfortranarray(np_flue.expm_su3(h * X) @ U)


@pytest.mark.parametrize("dims,eps,seed", [((4, 4, 4, 4), 0.4, 1), ((5, 3, 4, 3), 0.7, 2)])
def test_magnetic_force_vs_oracle(dims, eps, seed):
    U = generate.random_field(dims, eps, seed)
    b, g = forces.magnetic_force(U)
    assert abs(b - oracle.magnetic(U)) < 1e-12 * max(1, abs(b))
    go = oracle.loop5_energy_force(U, oracle.B2_PLANES)
    assert np.abs(_np(g) - go).max() < 1e-11 * max(1.0, np.abs(go).max())
    assert np.abs(_np(g)[..., 0, :, :]).max() == 0.0


def test_energy_force_all_planes_vs_oracle():
    U = generate.random_field((4, 3, 4, 5), 0.5, 3)
    e, g = forces.loop5_energy_force(U, forces.ALL_PLANES)
    assert abs(e - oracle.loop5_energy(U, oracle.ALL_PLANES)) < 1e-12 * abs(e)
    go = oracle.loop5_energy_force(U, oracle.ALL_PLANES)
    assert np.abs(_np(g) - go).max() < 1e-11 * np.abs(go).max()
    # plane orientation does not change the energy
    e2, g2 = forces.loop5_energy_force(U, ((2, 1), (3, 1), (4, 1), (3, 2), (4, 2), (4, 3)))
    assert abs(e2 - e) < 1e-12 * abs(e)
    assert np.abs(_np(g2) - _np(g)).max() < 1e-12


def test_plaquette_force_vs_staple():
    U = generate.random_field((4, 4, 3, 5), 0.6, 4)
    s, g = forces.plaquette_force(U)
    assert abs(s - oracle.plaquette(U, 1, 4, 4)[0]) < 1e-12 * abs(s)
    assert np.abs(_np(g) - oracle.plaquette_staple_force(U)).max() < 1e-12


def test_fd_along_random_directions_fp64():
    U = generate.random_field((8, 6, 6, 6), 0.3, 5)
    _, g = forces.magnetic_force(U)
    gn = _np(g)
    h = 1e-4
    worst = 0.0
    for k in range(8):
        X = generate.random_su3_algebra(U.shape[:5], 100 + k)
        fd = (G.magnetic(_perturb(U, X, h)) - G.magnetic(_perturb(U, X, -h))) / (2 * h)
        an = _lie_pair(gn, X)
        worst = max(worst, abs(an - fd) / abs(fd))
    assert worst < 1e-6


def test_euclid_form_and_autograd():
    U = generate.random_field((4, 4, 4, 4), 0.5, 6)
    _, gl = forces.magnetic_force(U, form="lie")
    _, ge = forces.magnetic_force(U, form="euclid")
    # Lie gradient from the Euclidean one: G = -1/2 TA(U N), N = Gamma^+
    m = U @ np_flue.dag(_np(ge))
    ah = 0.5 * (m - np_flue.dag(m))
    ta = ah - np.trace(ah, axis1=-2, axis2=-1)[..., None, None] * np.eye(3) / 3
    assert np.abs(-0.5 * ta - _np(gl)).max() < 1e-13
    # torch.autograd: directional derivative along a random complex direction
    Ut = torch.tensor(U, device="cuda", requires_grad=True)
    b = forces.magnetic_autograd(Ut)
    b.backward()
    D = np.random.default_rng(0).standard_normal(U.shape) * (1 + 1j)
    h = 1e-6
    fd = (G.magnetic(np.asfortranarray(U + h * D)) - G.magnetic(np.asfortranarray(U - h * D))) / (2 * h)
    an = float(np.sum((np.conj(_np(Ut.grad)) * D).real))
    assert abs(an - fd) < 1e-6 * abs(fd)


@pytest.mark.parametrize("prec", ["c64", "r12"])
def test_fp32_force_error_bound(prec):
    U = generate.random_field((8, 8, 8, 8), 0.3, 7)
    b64, g64 = forces.magnetic_force(U)
    b32, g32 = forces.magnetic_force(GaugeField.from_array(U, prec=prec))
    g64, g32 = _np(g64), _np(g32).astype(np.complex128)
    assert abs(b32 - b64) / abs(b64) < 1e-6
    assert np.linalg.norm(g32 - g64) / np.linalg.norm(g64) < 1e-6  # measured 2.2e-7 (c64, r12)


@pytest.mark.parametrize("pinned", [True, False])
def test_host_buffer_force_entry(pinned):
    """flue_magnetic_force_c: host complex64 in, host gradient out (zero-copy
    when the GPU can address the buffers, staged copies otherwise)."""
    import ctypes

    from flue_gb300 import _lib

    U = generate.random_field((8, 4, 6, 4), 0.4, 9)
    f = GaugeField.from_array(U, prec="c64")
    b_ref, g_ref = forces.magnetic_force(f)
    host = torch.as_tensor(np.asfortranarray(U.astype(np.complex64))).permute(6, 5, 4, 3, 2, 1, 0).contiguous()
    grad = torch.zeros_like(host)
    if pinned:
        host, grad = host.pin_memory(), grad.pin_memory()
    L = _lib.load()
    b = ctypes.c_double()
    nt, nx, ny, nz = U.shape[:4]
    for prec in (_lib.C64, _lib.R12):
        rc = L.flue_magnetic_force_c(ctypes.c_void_p(host.data_ptr()), _lib.C64, nt, nx, ny, nz, prec,
                                     _lib.FORCE_LIE, ctypes.byref(b), ctypes.c_void_p(grad.data_ptr()))
        assert rc == 0, L.flue_last_error_detail()
        assert abs(b.value - b_ref) < 1e-6 * abs(b_ref)
        g = grad.permute(6, 5, 4, 3, 2, 1, 0).numpy()
        assert np.abs(g - _np(g_ref)).max() < 1e-5 * np.abs(_np(g_ref)).max()


@pytest.mark.parametrize("prec_name,data_name", [("c64", "c64"), ("r12", "c64"), ("c128", "c128"), ("r12", "c128"),
                                                 ("c64", "c128")])
def test_host_buffer_force_time_slabs(prec_name, data_name, monkeypatch):
    """The host-buffer force pipelined over time slabs (even, uneven and
    one-slice slabs) gives the gradient of the single-pass call bit for bit
    and B^2 to FP64 summation order -- also for a complex128 field computed
    in FP32, whose gradient comes back as complex128 and equals the device
    FP32 gradient of the same field widened."""
    import ctypes

    from flue_gb300 import _lib

    U = generate.random_field((8, 4, 6, 4), 0.4, 10)
    c128 = data_name == "c128"
    dt = np.complex128 if c128 else np.complex64
    host = torch.as_tensor(np.asfortranarray(U.astype(dt))).permute(6, 5, 4, 3, 2, 1, 0).contiguous().pin_memory()
    L = _lib.load()
    code = {"c64": _lib.C64, "r12": _lib.R12, "c128": _lib.C128}[prec_name]
    src = _lib.C128 if c128 else _lib.C64

    def run(slabs):
        monkeypatch.setenv("FLUE_SLABS", str(slabs))
        grad = torch.full_like(host, float("nan")).pin_memory()
        b = ctypes.c_double()
        rc = L.flue_magnetic_force_c(ctypes.c_void_p(host.data_ptr()), src, 8, 4, 6, 4, code, _lib.FORCE_LIE,
                                     ctypes.byref(b), ctypes.c_void_p(grad.data_ptr()))
        assert rc == 0, L.flue_last_error_detail()
        return b.value, grad.numpy().copy()

    b1, g1 = run(1)
    assert np.isfinite(g1).all()
    if c128 and prec_name != "c128":
        bd, gd = forces.magnetic_force(GaugeField.from_array(U, prec=prec_name))
        assert abs(b1 - bd) < 1e-12 * abs(bd)
        assert np.array_equal(g1, _np(gd).astype(np.complex128).transpose(6, 5, 4, 3, 2, 1, 0))
    for slabs in (2, 3, 8):
        b, g = run(slabs)
        assert abs(b - b1) < 1e-12 * abs(b1), slabs
        assert np.array_equal(g, g1), slabs
    # the zero time-direction gradient written by the GPU instead of host threads
    monkeypatch.setenv("FLUE_HOST_ZERO", "0")
    b, g = run(3)
    assert np.array_equal(g, g1)
    monkeypatch.delenv("FLUE_HOST_ZERO")
    # B^2 alone (no gradient) through the pipeline
    monkeypatch.setenv("FLUE_SLABS", "4")
    b = ctypes.c_double()
    assert L.flue_magnetic_force_c(ctypes.c_void_p(host.data_ptr()), src, 8, 4, 6, 4, code, _lib.FORCE_LIE,
                                   ctypes.byref(b), None) == 0
    assert abs(b.value - b1) < 1e-12 * abs(b1)


@pytest.mark.parametrize("prec_name,data_name,slabs", [("r12", "c128", 10), ("r12", "c128", 14), ("c64", "c128", 10),
                                                       ("c128", "c128", 13), ("r12", "c64", 20), ("c64", "c64", 7)])
def test_host_buffer_force_dma_chunks(prec_name, data_name, slabs, monkeypatch):
    """Pinned host buffers move by copy-engine copies of time-slice chunks
    (FLUE_DMA_CHUNK slices rounded up to whole slabs; several chunks here, the
    last one short, slabs of uneven length): the field in after its first
    chunk, the gradient out before its last slabs (FLUE_OUT_TAIL of them, 0 =
    none).  Every mix of copies and kernel reads / writes gives the
    single-pass call's gradient bit for bit."""
    import ctypes

    from flue_gb300 import _lib

    dims = (40, 4, 6, 4)
    U = generate.random_field(dims, 0.4, 12)
    dt = np.complex128 if data_name == "c128" else np.complex64
    host = torch.as_tensor(np.asfortranarray(U.astype(dt))).permute(6, 5, 4, 3, 2, 1, 0).contiguous().pin_memory()
    L = _lib.load()
    code = {"c64": _lib.C64, "r12": _lib.R12, "c128": _lib.C128}[prec_name]
    src = _lib.C128 if data_name == "c128" else _lib.C64

    def run(nslab, dma_in, dma_out="1", tail="4", chunk="16"):
        monkeypatch.setenv("FLUE_SLABS", str(nslab))
        monkeypatch.setenv("FLUE_DMA_IN", dma_in)
        monkeypatch.setenv("FLUE_DMA_OUT", dma_out)
        monkeypatch.setenv("FLUE_OUT_TAIL", tail)
        monkeypatch.setenv("FLUE_DMA_CHUNK", chunk)
        grad = torch.full_like(host, float("nan")).pin_memory()
        b = ctypes.c_double()
        rc = L.flue_magnetic_force_c(ctypes.c_void_p(host.data_ptr()), src, *dims, code, _lib.FORCE_LIE,
                                     ctypes.byref(b), ctypes.c_void_p(grad.data_ptr()))
        assert rc == 0, L.flue_last_error_detail()
        return b.value, grad.numpy().copy()

    b1, g1 = run(1, "1")
    assert np.isfinite(g1).all()
    for mode in (("1", "1", "4"), ("1", "1", "0"), ("1", "1", "1"), ("0", "1", "2"), ("1", "0"), ("0", "0"),
                 ("1", "1", "2", "5"), ("1", "1", "0", "32")):
        b, g = run(slabs, *mode)
        assert np.array_equal(g, g1), mode
        assert abs(b - b1) < 1e-12 * abs(b1), mode


@pytest.mark.parametrize("slabs,streams", [(2, 2), (3, 4), (8, 3), (8, 1)])
def test_device_force_time_slabs(slabs, streams, monkeypatch):
    """The device B^2 force over time slabs on several streams equals the
    single-pass call: gradient bit for bit, B^2 to FP64 summation order; the
    same for B^2 alone and for a spatial-plane 5-loop energy."""
    U = generate.random_field((8, 4, 6, 5), 0.4, 11)
    f = GaugeField.from_array(U, prec="r12")
    monkeypatch.setenv("FLUE_SLABS", "1")
    b1, g1 = forces.magnetic_force(f)
    g1 = _np(g1).copy()
    m1 = G.magnetic(f)
    e1, h1 = forces.loop5_energy_force(f, ((3, 2), (4, 2)))
    h1 = _np(h1).copy()
    monkeypatch.setenv("FLUE_SLABS", str(slabs))
    monkeypatch.setenv("FLUE_SLAB_STREAMS", str(streams))
    b, g = forces.magnetic_force(f)
    assert abs(b - b1) < 1e-12 * abs(b1)
    assert np.array_equal(_np(g), g1)
    assert abs(G.magnetic(f) - m1) < 1e-12 * abs(m1)
    e, h = forces.loop5_energy_force(f, ((3, 2), (4, 2)))
    assert abs(e - e1) < 1e-12 * abs(e1)
    assert np.array_equal(_np(h), h1)


@pytest.mark.parametrize("copy_streams", ["1", "4"])
def test_host_buffer_force_staged_copies(copy_streams, monkeypatch):
    """With zero-copy turned off (FLUE_ZERO_COPY=0) the host-buffer force
    goes through library device buffers; a 127 MB field takes the chunked
    multi-stream copy path.  Its gradient equals the zero-copy pipeline's
    bit for bit, B^2 to FP64 summation order."""
    import ctypes

    from flue_gb300 import _lib

    dims = (32, 24, 24, 24)
    f = generate.random_field(dims, 0.3, 21, device="cuda")
    host = GaugeField.from_array(f, prec="c64").to_tensor(torch.complex64).permute(6, 5, 4, 3, 2, 1, 0)
    host = host.contiguous().cpu().pin_memory()
    assert host.numel() * 8 > 64 << 20
    L = _lib.load()

    def run():
        grad = torch.full_like(host, float("nan")).pin_memory()
        b = ctypes.c_double()
        rc = L.flue_magnetic_force_c(ctypes.c_void_p(host.data_ptr()), _lib.C64, *dims, _lib.R12, _lib.FORCE_LIE,
                                     ctypes.byref(b), ctypes.c_void_p(grad.data_ptr()))
        assert rc == 0, L.flue_last_error_detail()
        return b.value, grad

    b_zc, g_zc = run()
    monkeypatch.setenv("FLUE_ZERO_COPY", "0")
    monkeypatch.setenv("FLUE_COPY_STREAMS", copy_streams)
    b_st, g_st = run()
    L.flue_release_host_cache()
    assert abs(b_st - b_zc) < 1e-12 * abs(b_zc)
    assert torch.equal(g_st, g_zc)


def test_concurrent_host_threads(monkeypatch):
    """Four host threads computing B^2 forces of different fields at once (the
    time-slab path shares the library's streams and events between calls)
    get the same results as one thread in turn."""
    import threading

    monkeypatch.setenv("FLUE_SLABS", "4")
    Us = [generate.random_field((8, 4, 6, 4), 0.4, 60 + k) for k in range(4)]
    fs = [GaugeField.from_array(U, prec="r12") for U in Us]
    seq = [forces.magnetic_force(f) for f in fs]
    seq = [(b, _np(g).copy()) for b, g in seq]
    out = [None] * 4
    errs = []

    def work(k):
        try:
            s = torch.cuda.Stream()
            with torch.cuda.stream(s):
                b, g = forces.magnetic_force(fs[k])
                s.synchronize()
                out[k] = (b, _np(g).copy())
        except Exception as e:  # pragma: no cover - reported below
            errs.append(e)

    for _ in range(3):
        th = [threading.Thread(target=work, args=(k,)) for k in range(4)]
        for t in th:
            t.start()
        for t in th:
            t.join()
        assert not errs, errs
        for (b, g), (bs, gs) in zip(out, seq):
            assert abs(b - bs) < 1e-12 * abs(bs)
            assert np.array_equal(g, gs)


@pytest.mark.parametrize("dt,code,src", [(np.complex64, "r12", "c64"), (np.complex128, "c128", "c128")])
def test_host_buffer_misaligned_input(dt, code, src, monkeypatch):
    """A host field 16 bytes past a 64-byte boundary (as numpy's allocator
    places large arrays) takes the shifted slab schedule; its B^2 and
    gradient equal those of an aligned copy, bit for bit for the gradient."""
    import ctypes

    from flue_gb300 import _lib

    monkeypatch.setenv("FLUE_SLABS", "4")
    dims = (16, 4, 6, 4)
    U = generate.random_field(dims, 0.4, 23).astype(dt)
    n = U.size
    esz = np.dtype(dt).itemsize
    buf = np.zeros(n + 64 // esz * 2, dtype=dt)
    off = ((16 - buf.ctypes.data % 64) % 64) // esz
    mis = buf[off:off + n].reshape(U.shape, order="F")
    mis[...] = U
    assert mis.ctypes.data % 64 == 16
    L = _lib.load()
    codes = {"r12": _lib.R12, "c128": _lib.C128}
    srcs = {"c64": _lib.C64, "c128": _lib.C128}

    def run(arr):
        g = np.zeros(U.shape, dtype=dt, order="F")
        b = ctypes.c_double()
        rc = L.flue_magnetic_force_c(ctypes.c_void_p(arr.ctypes.data), srcs[src], *dims, codes[code], _lib.FORCE_LIE,
                                     ctypes.byref(b), ctypes.c_void_p(g.ctypes.data))
        assert rc == 0, L.flue_last_error_detail()
        return b.value, g

    b1, g1 = run(np.asfortranarray(U))
    b2, g2 = run(mis)
    assert abs(b2 - b1) < 1e-12 * abs(b1)
    assert np.array_equal(g2, g1)


@pytest.mark.parametrize("prec", ["c64", "r12"])
def test_forward_tile_variant(prec, monkeypatch):
    """The forward with the lines staged per timeslice tile in shared memory
    (FLUE_FWD_TILE=1: 2 time slices x 8 x 8 patches, cp.async) against the
    default forward (lines read through L1/L2) and the oracle: B^2 alone, B^2
    and its gradient, in one pass and in time slabs; a lattice the tiles do
    not fit falls back to the default kernel."""
    U = generate.random_field((4, 8, 8, 16), 0.4, 21)
    bo = oracle.magnetic(U)
    go = oracle.loop5_energy_force(U, oracle.B2_PLANES)
    f = GaugeField.from_array(U, prec=prec)
    monkeypatch.setenv("FLUE_FWD_TILE", "0")
    b0, g0 = forces.magnetic_force(f)
    g0 = _np(g0).copy()
    m0 = G.magnetic(f)
    monkeypatch.setenv("FLUE_FWD_TILE", "1")
    for slabs in ("1", "2"):
        monkeypatch.setenv("FLUE_SLABS", slabs)
        b1, g1 = forces.magnetic_force(f)
        g1 = _np(g1).astype(np.complex128)
        assert abs(b1 - b0) < 1e-6 * abs(b0)
        assert abs(G.magnetic(f) - m0) < 1e-6 * abs(m0)
        assert np.linalg.norm(g1 - g0) < 1e-6 * np.linalg.norm(g0)
        assert abs(b1 - bo) < 1e-6 * abs(bo)
        assert np.linalg.norm(g1 - go) < 1e-6 * np.linalg.norm(go)
    U2 = generate.random_field((4, 6, 8, 8), 0.4, 22)  # NX = 6: no 8 x 8 patch in the planes with x
    b2 = G.magnetic(GaugeField.from_array(U2, prec=prec))
    assert abs(b2 - oracle.magnetic(U2)) < 1e-6 * abs(oracle.magnetic(U2))
