"""Host-side grid geometry: the reference's wavenumber tables and the kept
(non-dealiased) mode bounds.

``wavenumbers`` reproduces ``FourierRepresentation._setup_k``
(dedalus/data_objects/representations.py:204-233) exactly, including the
Nyquist sign flip, so the device sees the same float64 k values the reference
multiplies by.  ``kept_bounds`` evaluates the reference's own dealias test
(``|k_i| >= 2/3 kny_i`` zeroed, representations.py:384-397 and
dealias_cy_3d.pyx:34-37; ``|k_i| == kny_i`` for the 'None' method,
representations.py:442-455) and turns the kept set of each axis into its
largest kept mode index m, checking that it is the symmetric low band the
kernels prune to.
"""
import numpy as np
import numpy.fft as npfft


def swap_indices(arr):
    """dedalus/utils/parallelism.py:155-173."""
    out = list(arr) if isinstance(arr, (list, tuple)) else np.array(arr, copy=True)
    out[0], out[1] = out[1], out[0]
    return out


def kspace_shape(xshape):
    ks = list(xshape)
    ks[-1] = ks[-1] // 2 + 1
    return tuple(swap_indices(ks))


def wavenumbers(xshape, length):
    """Return (k dict of broadcastable arrays, kny in k-layout order, ktrans)."""
    xshape = np.array(xshape)
    length = np.asarray(length, dtype=np.float64)
    ndim = len(xshape)
    if ndim == 2:
        ktrans = {'x': 0, 0: 'x', 'y': 1, 1: 'y'}
    else:
        ktrans = {'x': 2, 2: 'x', 'y': 0, 0: 'y', 'z': 1, 1: 'z'}
    kshape = kspace_shape(list(xshape))
    kny = swap_indices(np.pi * xshape / length)
    rcomp = ktrans['x']
    k = {}
    for i, ksize in enumerate(kshape):
        xsize = swap_indices(xshape)[i]
        if i == rcomp:
            ki = npfft.fftfreq(xsize)[:ksize] * 2. * kny[i]
            if xsize % 2 == 0:
                ki[-1] *= -1.
        else:
            ki = npfft.fftfreq(ksize) * 2. * kny[i]
            if xsize % 2 == 0:
                ki[ksize // 2] *= -1.
        k[ktrans[i]] = ki.reshape(i * (1,) + (ksize,) + (ndim - i - 1) * (1,))
    return k, np.asarray(kny, dtype=np.float64), ktrans


def _axis_kept(kvals, kny_i, method):
    a = np.abs(np.asarray(kvals).reshape(-1))
    if method in ('2/3', '2/3 cython'):
        # dealias_cy_3d.pyx:34: zeroed if k >= 2/3*kny or k <= -2/3*kny
        t = 2. / 3. * kny_i
        kv = np.asarray(kvals).reshape(-1)
        return ~((kv >= t) | (kv <= -t))
    if method in ('None', None, 0):
        return ~(a == kny_i)
    raise NotImplementedError("dealiasing method %r is not supported by the CUDA path" % (method,))


def kept_bounds(xshape, length, method='2/3 cython'):
    """Largest kept |mode index| per axis, as (mx, my, mz) (mz = 0 in 2D)."""
    k, kny, ktrans = wavenumbers(xshape, length)
    ndim = len(xshape)
    out = {}
    for name in ('x', 'y', 'z')[:ndim]:
        i = ktrans[name]
        kept = _axis_kept(k[name], kny[i], method)
        n = kept.size
        if name == 'x':
            m = int(np.argmin(kept)) - 1 if not kept.all() else n - 1
            expect = np.arange(n) <= m
        else:
            # full axis: kept must be [0, m] U [n-m, n)
            m = int(np.argmin(kept[: n // 2 + 1])) - 1 if not kept[: n // 2 + 1].all() else n // 2
            idx = np.arange(n)
            expect = (idx <= m) | (idx >= n - m)
        if m < 0 or not np.array_equal(kept, expect):
            raise NotImplementedError("the dealias mask along %s is not a symmetric low band" % name)
        out[name] = m
    return out['x'], out['y'], out.get('z', 0)


def k_tables(xshape, length):
    """1-D float64 k tables in plan order: (kx[Nx/2+1], ky[Ny], kz[Nz] or None)."""
    k, _, _ = wavenumbers(xshape, length)
    kx = np.ascontiguousarray(k['x'].reshape(-1))
    ky = np.ascontiguousarray(k['y'].reshape(-1))
    kz = np.ascontiguousarray(k['z'].reshape(-1)) if 'z' in k else None
    return kx, ky, kz


def integer_k(xshape, length):
    """True when every wavenumber is an exact integer (length 2 pi axes)."""
    for t in k_tables(xshape, length):
        if t is not None and not np.array_equal(t, np.round(t)):
            return False
    return True
