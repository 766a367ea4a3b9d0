"""CPU oracle -- test infrastructure only.

ctypes front end for ``oracle/stage.c``, the plain-C restatement of the
reference's Cython stage kernels (``forward_step_cy_{2d,3d}.pyx``) and dealias
kernels (``dealias_cy_{2d,3d}.pyx``).  The wrappers take the reference's own
argument orders:

* ``euler(start, output, deriv, dt)``               forward_step_cy_3d.pyx:17
* ``etd1(start, output, deriv, intfactor, dt)``       forward_step_cy_3d.pyx:34
* ``etd2rk1/etd2rk2(start, output, deriv1, deriv2, intfactor, dt)``  :63, :95
* ``dealias_23(data, kx, ky[, kz], knyquist)``        dealias_cy_3d.pyx:13

Like the Cython originals they require contiguous complex128 arrays of one
shape (float64 for ``intfactor``) and raise ``ValueError`` otherwise.
"""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "stage.c")
LIB = os.path.join(HERE, "libddoracle.so")

_lib = None


def build(force=False):
    """Compile stage.c with gcc (no FMA contraction) into oracle/libddoracle.so."""
    if force or not os.path.isfile(LIB) or os.path.getmtime(LIB) < os.path.getmtime(SRC):
        tmp = LIB + ".tmp%d" % os.getpid()
        subprocess.check_call(["gcc", "-O2", "-ffp-contract=off", "-fPIC", "-shared",
                               SRC, "-o", tmp, "-lm"])
        os.replace(tmp, LIB)
    return LIB


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(LIB)
        P = ctypes.c_void_p
        D = ctypes.c_double
        I = ctypes.c_int
        N = ctypes.c_int64
        L.dd_oracle_euler.argtypes = [P, P, P, D, N]
        L.dd_oracle_etd1.argtypes = [I, P, P, P, P, D, N]
        L.dd_oracle_etd2rk1.argtypes = [I, P, P, P, P, P, D, N]
        L.dd_oracle_etd2rk2.argtypes = [I, P, P, P, P, P, D, N]
        L.dd_oracle_dealias_23_3d.argtypes = [P, P, I, P, I, P, I, P]
        L.dd_oracle_dealias_23_2d.argtypes = [P, P, I, P, I, P]
        for f in (L.dd_oracle_euler, L.dd_oracle_etd1, L.dd_oracle_etd2rk1,
                  L.dd_oracle_etd2rk2, L.dd_oracle_dealias_23_3d, L.dd_oracle_dealias_23_2d):
            f.restype = None
        _lib = L
    return _lib


def _c128(a, shape=None):
    if not isinstance(a, np.ndarray) or a.dtype != np.complex128 or not a.flags.c_contiguous:
        raise ValueError("Buffer dtype mismatch: expected contiguous complex128")
    if shape is not None and a.shape != shape:
        raise ValueError("Buffer shape mismatch")
    return a.ctypes.data


def _f64(a, shape):
    if not isinstance(a, np.ndarray) or a.dtype != np.float64 or not a.flags.c_contiguous:
        raise ValueError("Buffer dtype mismatch: expected contiguous float64")
    if a.shape != shape:
        raise ValueError("Buffer shape mismatch")
    return a.ctypes.data


class StageKernels:
    """The four stage kernels for one dimensionality (2 or 3)."""

    def __init__(self, ndim):
        if ndim not in (2, 3):
            raise ValueError("ndim must be 2 or 3")
        self.ndim = ndim

    def _check(self, start):
        if start.ndim != self.ndim:
            raise ValueError("Buffer has wrong number of dimensions (expected %d, got %d)"
                             % (self.ndim, start.ndim))

    def euler(self, start, output, deriv, dt):
        self._check(start)
        s = start.shape
        lib().dd_oracle_euler(_c128(start), _c128(output, s), _c128(deriv, s), float(dt), start.size)

    def etd1(self, start, output, deriv, intfactor, dt):
        self._check(start)
        s = start.shape
        lib().dd_oracle_etd1(self.ndim, _c128(start), _c128(output, s), _c128(deriv, s),
                             _f64(intfactor, s), float(dt), start.size)

    def etd2rk1(self, start, output, deriv1, deriv2, intfactor, dt):
        self._check(start)
        s = start.shape
        lib().dd_oracle_etd2rk1(self.ndim, _c128(start), _c128(output, s), _c128(deriv1, s),
                                _c128(deriv2, s), _f64(intfactor, s), float(dt), start.size)

    def etd2rk2(self, start, output, deriv1, deriv2, intfactor, dt):
        self._check(start)
        s = start.shape
        lib().dd_oracle_etd2rk2(self.ndim, _c128(start), _c128(output, s), _c128(deriv1, s),
                                _c128(deriv2, s), _f64(intfactor, s), float(dt), start.size)


stage2d = StageKernels(2)
stage3d = StageKernels(3)


def dealias_23(data, kx, ky, *rest):
    """dealias_23(data, kx, ky[, kz], knyquist) with the reference's broadcast k arrays."""
    if data.ndim == 3:
        kz, knyquist = rest
        kxv = np.ascontiguousarray(np.asarray(kx, dtype=np.float64).reshape(-1))
        kyv = np.ascontiguousarray(np.asarray(ky, dtype=np.float64).reshape(-1))
        kzv = np.ascontiguousarray(np.asarray(kz, dtype=np.float64).reshape(-1))
        kn = np.ascontiguousarray(knyquist, dtype=np.float64)
        ny, nz, nx = data.shape
        if kxv.size != nx or kyv.size != ny or kzv.size != nz:
            raise ValueError("k array sizes do not match data")
        lib().dd_oracle_dealias_23_3d(_c128(data), kxv.ctypes.data, nx, kyv.ctypes.data, ny,
                                      kzv.ctypes.data, nz, kn.ctypes.data)
    elif data.ndim == 2:
        (knyquist,) = rest
        kxv = np.ascontiguousarray(np.asarray(kx, dtype=np.float64).reshape(-1))
        kyv = np.ascontiguousarray(np.asarray(ky, dtype=np.float64).reshape(-1))
        kn = np.ascontiguousarray(knyquist, dtype=np.float64)
        nx, ny = data.shape
        if kxv.size != nx or kyv.size != ny:
            raise ValueError("k array sizes do not match data")
        lib().dd_oracle_dealias_23_2d(_c128(data), kxv.ctypes.data, nx, kyv.ctypes.data, ny,
                                      kn.ctypes.data)
    else:
        raise ValueError("data must be 2D or 3D")
