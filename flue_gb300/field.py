"""Device-resident gauge fields.

A :class:`GaugeField` owns (or wraps) a CUDA tensor holding the links in one
of the device layouts of include/flue_gb300.h:

* ``"c128"`` / ``"c64"``: the reference's own Fortran-ordered array
  ``data(NT,NX,NY,NZ,4,3,3)`` (src/wloops.F90:60), i.e. a contiguous torch
  tensor of shape ``(3,3,4,NZ,NY,NX,NT)`` -- site-fastest
  structure-of-arrays.  A Fortran-ordered numpy array or a tensor with those
  strides is used without any re-layout.
* ``"r12"``: reconstruct-12 FP32, a float32 tensor ``(4,3,NZ,NY,NX,NT,4)``.

``c128`` fields are computed in FP64; ``c64`` and ``r12`` in FP32 with FP64
global sums.
"""
from __future__ import annotations

import collections
import ctypes
from typing import Tuple

import numpy as np
import torch

from . import _lib

PRECS = {"c128": _lib.C128, "c64": _lib.C64, "r12": _lib.R12}
_PREC_NAMES = {v: k for k, v in PRECS.items()}


def _require_cuda():
    if not torch.cuda.is_available():
        raise RuntimeError("flue_gb300 needs a CUDA device; no CPU fallback exists")


def _stream_handle():
    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)


def _ptr(t: torch.Tensor):
    return ctypes.c_void_p(t.data_ptr())


class Workspace:
    """Scratch buffers reused across calls (allocated by torch), one per
    (device, stream): calls queued on the same stream run in order and can
    share one, calls on different streams may run at once and must not.
    At most MAX_ENTRIES buffers are kept, the least recently used dropped
    first; torch hands a dropped buffer's memory only to later allocations on
    the same stream, so work still queued with it is unaffected."""

    MAX_ENTRIES = 8
    _bufs = collections.OrderedDict()

    @classmethod
    def get(cls, nbytes: int, device) -> torch.Tensor:
        dev = torch.device(device)
        idx = dev.index if dev.index is not None else torch.cuda.current_device()
        key = (idx, torch.cuda.current_stream(idx).cuda_stream)
        buf = cls._bufs.pop(key, None)
        if buf is None or buf.numel() < nbytes:
            buf = torch.empty(max(int(nbytes), 256), dtype=torch.uint8, device=torch.device("cuda", idx))
        cls._bufs[key] = buf
        while len(cls._bufs) > cls.MAX_ENTRIES:
            cls._bufs.popitem(last=False)
        return buf

    @classmethod
    def release(cls):
        cls._bufs.clear()


class GaugeField:
    """Links of an SU(3) gauge field on a periodic NT x NX x NY x NZ lattice."""

    def __init__(self, storage: torch.Tensor, dims: Tuple[int, int, int, int], prec: str):
        if prec not in PRECS:
            raise ValueError(f"prec must be one of {sorted(PRECS)}")
        if not storage.is_cuda:
            raise ValueError("GaugeField storage must live on a CUDA device")
        self.storage = storage
        self.dims = tuple(int(d) for d in dims)
        self.prec = prec

    # ------------------------------------------------------------------
    @property
    def nt(self):
        return self.dims[0]

    @property
    def volume(self) -> int:
        nt, nx, ny, nz = self.dims
        return nt * nx * ny * nz

    @property
    def device(self):
        return self.storage.device

    @property
    def compute_dtype(self):
        return torch.complex128 if self.prec == "c128" else torch.complex64

    def descriptor(self) -> _lib.FlueField:
        nt, nx, ny, nz = self.dims
        return _lib.FlueField(self.storage.data_ptr(), nt, nx, ny, nz, PRECS[self.prec])

    def nbytes(self) -> int:
        return int(self.storage.numel() * self.storage.element_size())

    # ------------------------------------------------------------------
    @classmethod
    def empty(cls, dims, prec="c128", device="cuda"):
        _require_cuda()
        nt, nx, ny, nz = dims
        if prec == "c128":
            st = torch.empty((3, 3, 4, nz, ny, nx, nt), dtype=torch.complex128, device=device)
        elif prec == "c64":
            st = torch.empty((3, 3, 4, nz, ny, nx, nt), dtype=torch.complex64, device=device)
        else:
            st = torch.empty((4, 3, nz, ny, nx, nt, 4), dtype=torch.float32, device=device)
        return cls(st, dims, prec)

    @classmethod
    def from_array(cls, data, prec: str | None = None, reunitarise: bool = False, device=None) -> "GaugeField":
        """Build a device field from ``data[t,x,y,z,mu,a,b]`` (numpy or torch,
        complex128 or complex64, any strides).  ``prec`` defaults to the
        input's own precision.  Fortran-ordered inputs whose precision already
        matches are used without re-layout (a CUDA tensor is wrapped, not
        copied)."""
        _require_cuda()
        if isinstance(data, GaugeField):
            if (prec is None or prec == data.prec) and not reunitarise:
                return data
            data = data.to_tensor()
        t = torch.as_tensor(data) if not isinstance(data, torch.Tensor) else data
        if t.dim() != 7 or tuple(t.shape[4:]) != (4, 3, 3):
            raise ValueError(f"gauge field must have shape (NT,NX,NY,NZ,4,3,3), got {tuple(t.shape)}")
        if t.dtype not in (torch.complex128, torch.complex64):
            raise TypeError(f"gauge field must be complex128 or complex64, got {t.dtype}")
        if prec is None:
            prec = "c128" if t.dtype == torch.complex128 else "c64"
        if prec not in PRECS:
            raise ValueError(f"prec must be one of {sorted(PRECS)}")
        dims = tuple(int(d) for d in t.shape[:4])
        dev = torch.device(device) if device is not None else (t.device if t.is_cuda else torch.device("cuda"))
        want_dtype = {"c128": torch.complex128, "c64": torch.complex64}.get(prec)
        # fast path: already the device layout and dtype
        ft = t.permute(6, 5, 4, 3, 2, 1, 0)
        if want_dtype is not None and t.dtype == want_dtype and ft.is_contiguous() and not reunitarise:
            st = ft if (t.is_cuda and t.device == dev) else ft.to(dev, non_blocking=False)
            return cls(st, dims, prec)
        # general path: copy the raw elements to the device once, then re-layout
        if t.is_cuda and t.device == dev:
            src = t
        else:
            if ft.is_contiguous():
                src = ft.to(dev).permute(6, 5, 4, 3, 2, 1, 0)
            else:
                src = t.contiguous().to(dev)
        out = cls.empty(dims, prec, dev)
        strides = (ctypes.c_int64 * 7)(*[int(s) for s in src.stride()])
        src_dtype = _lib.C128 if src.dtype == torch.complex128 else _lib.C64
        with torch.cuda.device(dev):
            _lib.call("flue_pack_field", _ptr(src), src_dtype, strides, *dims, _ptr(out.storage), PRECS[prec],
                      int(bool(reunitarise)), _stream_handle())
        return out

    def to_tensor(self, dtype=None) -> torch.Tensor:
        """The links as a CUDA tensor indexed [t,x,y,z,mu,a,b] (a view for
        c128/c64 fields, an expanded copy for r12)."""
        if dtype is None:
            dtype = self.compute_dtype
        if self.prec in ("c128", "c64") and dtype == self.compute_dtype:
            return self.storage.permute(6, 5, 4, 3, 2, 1, 0)
        nt, nx, ny, nz = self.dims
        out = torch.empty((3, 3, 4, nz, ny, nx, nt), dtype=dtype, device=self.device)
        d = self.descriptor()
        with torch.cuda.device(self.device):
            _lib.call("flue_unpack_field", ctypes.byref(d), _ptr(out),
                      _lib.C128 if dtype == torch.complex128 else _lib.C64, _stream_handle())
        return out.permute(6, 5, 4, 3, 2, 1, 0)

    def to_numpy(self) -> np.ndarray:
        """Host copy, complex128, Fortran-ordered (the reference's layout)."""
        t = self.to_tensor(torch.complex128)
        return np.asfortranarray(t.cpu().numpy())

    def clone(self) -> "GaugeField":
        return GaugeField(self.storage.clone(), self.dims, self.prec)

    def reunitarise_(self) -> "GaugeField":
        d = self.descriptor()
        with torch.cuda.device(self.device):
            _lib.call("flue_reunitarise_field", ctypes.byref(d), _stream_handle())
        return self

    def __repr__(self):
        return f"GaugeField(dims={self.dims}, prec={self.prec!r}, device={self.device})"


def as_field(data, prec: str | None = None) -> GaugeField:
    if isinstance(data, GaugeField) and (prec is None or prec == data.prec):
        return data
    return GaugeField.from_array(data, prec=prec)


def workspace(op: int, field: GaugeField) -> torch.Tensor:
    # the library launches on the calling thread's current device and stream
    cur = torch.cuda.current_device()
    if field.device.index != cur:
        raise ValueError(f"field lives on {field.device} but the current device is cuda:{cur}; "
                         f"call under torch.cuda.device({field.device.index})")
    nt, nx, ny, nz = field.dims
    n = _lib.load().flue_workspace_bytes(op, nt, nx, ny, nz, PRECS[field.prec])
    return Workspace.get(n, field.device)
