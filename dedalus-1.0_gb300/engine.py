"""Device-side plan objects: a grid geometry (``dd_plan``) plus a workspace
cache, shared by every field component of one representation.

Device memory comes from PyTorch; the C library only sees raw pointers and
the current torch CUDA stream.
"""
import ctypes
import threading

import numpy as np
import torch

from . import _lib
from . import kgrid


def current_stream():
    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)


def dptr(t):
    return ctypes.c_void_p(t.data_ptr())


class Plan:
    """One dd_plan for an (xshape, length, dealiasing) geometry."""

    def __init__(self, xshape, length, dealiasing='2/3 cython', device=None):
        self.xshape = tuple(int(n) for n in xshape)
        self.ndim = len(self.xshape)
        if self.ndim not in (2, 3):
            raise ValueError("Must use either 2 or 3 dimensions.")
        self.length = tuple(float(l) for l in length)
        self.dealiasing = dealiasing
        self.device = torch.device('cuda', torch.cuda.current_device() if device is None else device)
        self.kshape = kgrid.kspace_shape(list(self.xshape))
        self.mx, self.my, self.mz = kgrid.kept_bounds(self.xshape, self.length, dealiasing)
        self.kx, self.ky, self.kz = kgrid.k_tables(self.xshape, self.length)
        self.integer_k = kgrid.integer_k(self.xshape, self.length)
        shape = (ctypes.c_int64 * self.ndim)(*self.xshape)
        h = ctypes.c_void_p()
        with torch.cuda.device(self.device):
            _lib.call("dd_plan_create", self.ndim, shape,
                      self.kx.ctypes.data_as(ctypes.c_void_p), self.ky.ctypes.data_as(ctypes.c_void_p),
                      None if self.kz is None else self.kz.ctypes.data_as(ctypes.c_void_p),
                      self.mx, self.my, self.mz, ctypes.byref(h))
        self.handle = h
        self._ws = {}
        self._lock = threading.Lock()

    def __del__(self):
        h = getattr(self, 'handle', None)
        if h is not None and h.value:
            try:
                _lib.lib().dd_plan_destroy(h)
            except Exception:
                pass
            self.handle = None

    # --------------------------------------------------------------- sizes
    @property
    def kept(self):
        if self.ndim == 3:
            return (self.mx + 1, 2 * self.my + 1, 2 * self.mz + 1)
        return (self.mx + 1, 2 * self.my + 1)

    def workspace_bytes(self, nfield, precision=_lib.DD_FP64):
        n = ctypes.c_size_t()
        _lib.call("dd_plan_workspace_size", self.handle, nfield, precision, ctypes.byref(n))
        return n.value

    def workspace(self, nbytes, tag=0):
        """Cached uint8 device buffer of at least nbytes (per tag)."""
        with self._lock:
            buf = self._ws.get(tag)
            if buf is None or buf.numel() < nbytes:
                buf = torch.empty(max(int(nbytes), 16), dtype=torch.uint8, device=self.device)
                self._ws[tag] = buf
            return buf

    # ---------------------------------------------------------- transforms
    def r2c(self, xs, ks, precision=_lib.DD_FP64):
        """Forward transforms (x -> k, /N, dealiased) of lists of tensors."""
        nb = self.workspace_bytes(len(xs), precision)
        ws = self.workspace(nb)
        xp, _a = _lib.ptr_array([x.data_ptr() for x in xs])
        kp, _b = _lib.ptr_array([k.data_ptr() for k in ks])
        _lib.call("dd_fft_r2c", self.handle, len(xs), xp, kp, precision, dptr(ws), ws.numel(),
                  current_stream())

    def c2r(self, ks, xs, precision=_lib.DD_FP64):
        """Backward transforms (k -> x) of the kept modes."""
        nb = self.workspace_bytes(len(ks), precision)
        ws = self.workspace(nb)
        kp, _a = _lib.ptr_array([k.data_ptr() for k in ks])
        xp, _b = _lib.ptr_array([x.data_ptr() for x in xs])
        _lib.call("dd_fft_c2r", self.handle, len(ks), kp, xp, precision, dptr(ws), ws.numel(),
                  current_stream())

    def dealias(self, k):
        _lib.call("dd_dealias", self.handle, dptr(k), current_stream())

    # ------------------------------------------------ shearing-box transforms
    def _shear_ws(self, nfield):
        n = ctypes.c_size_t()
        _lib.call("dd_shear_workspace_size", self.handle, nfield, ctypes.byref(n))
        return self.workspace(n.value, tag='shear')

    def shear_r2c(self, xs, ks, kys, cut, pr, t):
        """Shearing-box forward transforms at time t (kys: sheared k_y table,
        pr: phase-rate table, both device float64)."""
        ws = self._shear_ws(len(xs))
        xp, _a = _lib.ptr_array([x.data_ptr() for x in xs])
        kp, _b = _lib.ptr_array([k.data_ptr() for k in ks])
        _lib.call("dd_shear_r2c", self.handle, len(xs), xp, kp, dptr(kys), float(cut), dptr(pr), float(t),
                  dptr(ws), ws.numel(), current_stream())

    def shear_c2r(self, ks, xs, kys, cut, pr, t):
        """Shearing-box backward transforms at time t."""
        ws = self._shear_ws(len(ks))
        kp, _a = _lib.ptr_array([k.data_ptr() for k in ks])
        xp, _b = _lib.ptr_array([x.data_ptr() for x in xs])
        _lib.call("dd_shear_c2r", self.handle, len(ks), kp, xp, dptr(kys), float(cut), dptr(pr), float(t),
                  dptr(ws), ws.numel(), current_stream())

    def shear_dealias(self, ks, kys, cut):
        kp, _a = _lib.ptr_array([k.data_ptr() for k in ks])
        _lib.call("dd_shear_dealias", self.handle, len(ks), kp, dptr(kys), float(cut), current_stream())


_PLANS = {}


def get_plan(xshape, length, dealiasing='2/3 cython'):
    """Shared plan per geometry and device (plans hold no per-field state)."""
    key = (tuple(int(n) for n in xshape), tuple(float(l) for l in length), str(dealiasing),
           torch.cuda.current_device())
    p = _PLANS.get(key)
    if p is None:
        p = Plan(xshape, length, dealiasing)
        _PLANS[key] = p
    return p
