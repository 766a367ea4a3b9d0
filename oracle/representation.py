"""CPU oracle -- test infrastructure only (never imported by the product path).

Python 3 restatement of the reference's ``FourierRepresentation``
(``dedalus/data_objects/representations.py:57-557``) on its numpy FFT
branch (``FFT.method = numpy``).  Layout, wavenumbers, the lazy x/k space
switch, normalisation and the 2/3 dealiasing rule follow the reference line by
line; only Python 2 idioms are updated (integer division, list-of-slices
indexing).  The '2/3 cython' dealias method calls the C restatement of the
reference's Cython kernel (``oracle/stage.c``).
"""
import configparser

import numpy as np
import numpy.fft as npfft

from . import _cstage

# Threads for the FFTs when timing the CPU baseline.  1 = numpy.fft exactly as
# the reference's FFT.method = numpy; > 1 = the same pocketfft algorithm
# through scipy.fft with that many workers (timing only, never in parity tests).
FFT_WORKERS = 1

# dedalus/config.py:29-53 (the keys the hot path reads)
decfg = configparser.ConfigParser()
decfg.add_section('FFT')
decfg.set('FFT', 'method', 'numpy')
decfg.set('FFT', 'dealiasing', '2/3 cython')
decfg.add_section('physics')
decfg.set('physics', 'use_tracer', 'False')
decfg.set('physics', 'boussinesq_direction', 'z')


def swap_indices(arr):
    """dedalus/utils/parallelism.py:155-173: swap entries [0] and [1]."""
    if isinstance(arr, np.ndarray):
        out_arr = arr.copy()
    elif isinstance(arr, list):
        out_arr = list(arr)
    else:
        raise NotImplementedError("swap_indices only implemented for numpy arrays and lists.")
    a = out_arr[1]
    out_arr[1] = out_arr[0]
    out_arr[0] = a
    return out_arr


class FourierRepresentation:
    """representations.py:57-557 (numpy FFT branch, single process)."""

    _static_k = True

    def __init__(self, sd, shape, length):
        # representations.py:97-136
        self.sd = sd
        self.global_shape = {'xspace': np.array(shape)}
        self.length = np.asarray(length, dtype=np.float64)
        self.ndim = len(shape)
        if self.ndim not in (2, 3):
            raise ValueError("Must use either 2 or 3 dimensions.")
        if len(shape) != len(length):
            raise ValueError("Shape and Length must have same dimensions.")
        self.dtype = {'kspace': 'complex128', 'xspace': 'float64'}
        self._eps = {'kspace': np.finfo(self.dtype['kspace']).eps,
                     'xspace': np.finfo(self.dtype['xspace']).eps}
        method = decfg.get('FFT', 'method')
        dealiasing = decfg.get('FFT', 'dealiasing')
        if self.ndim == 2:
            self.ktrans = {'x': 0, 0: 'x', 'y': 1, 1: 'y'}
            self.xtrans = {'x': 1, 1: 'x', 'y': 0, 0: 'y'}
        else:
            self.ktrans = {'x': 2, 2: 'x', 'y': 0, 0: 'y', 'z': 1, 1: 'z'}
            self.xtrans = {'x': 2, 2: 'x', 'y': 1, 1: 'y', 'z': 0, 0: 'z'}
        self.set_fft(method)
        self.set_dealiasing(dealiasing)
        self._setup_k()
        self._curr_space = 'kspace'
        self.data = self.kdata
        self.fwd_count = 0
        self.rev_count = 0

    def __getitem__(self, space):
        self.require_space(space)
        return self.data

    def __setitem__(self, space, data):
        # representations.py:144-166
        if space == 'xspace':
            self.data = self.xdata
        elif space == 'kspace':
            self.data = self.kdata
        else:
            raise KeyError("space must be either xspace or kspace.")
        if type(data) == float or type(data) == complex:
            self.data[:] = data
        else:
            sli = tuple(slice(i) for i in self.data.shape)
            self.data[:] = data[sli]
        self._curr_space = space

    def _allocate_memory(self, method):
        # representations.py:170-199, numpy branch
        self.global_shape['kspace'] = self.global_shape['xspace'].copy()
        self.global_shape['kspace'][-1] = self.global_shape['kspace'][-1] // 2 + 1
        self.global_shape['kspace'] = swap_indices(self.global_shape['kspace'])
        if method != 'numpy':
            raise NotImplementedError("The oracle implements the numpy FFT path only.")
        self.kdata = np.zeros(tuple(self.global_shape['kspace']), dtype=self.dtype['kspace'])
        self.xdata = np.zeros(tuple(self.global_shape['xspace']), dtype=self.dtype['xspace'])
        self.local_shape = {'kspace': self.global_shape['kspace'].copy(),
                            'xspace': self.global_shape['xspace'].copy()}
        self.offset = {'xspace': 0, 'kspace': 0}
        self.deriv_data = np.zeros_like(self.kdata)

    def _setup_k(self):
        # representations.py:204-233
        self.dk = 2 * np.pi / self.length
        self.dk = swap_indices(self.dk)
        self.kny = np.pi * self.global_shape['xspace'] / self.length
        self.kny = swap_indices(self.kny)
        rcomp = self.ktrans['x']
        self.k = {}
        for i, ksize in enumerate(self.global_shape['kspace']):
            xsize = swap_indices(self.global_shape['xspace'])[i]
            if i == rcomp:
                ki = npfft.fftfreq(xsize)[:ksize] * 2. * self.kny[i]
                if xsize % 2 == 0:
                    ki[-1] *= -1.
            else:
                ki = npfft.fftfreq(ksize) * 2. * self.kny[i]
                if xsize % 2 == 0:
                    ki[ksize // 2] *= -1.
            kshape = i * (1,) + (ksize,) + (self.ndim - i - 1) * (1,)
            ki = ki.reshape(kshape)
            self.k[self.ktrans[i]] = ki

    def require_space(self, space):
        if self._curr_space == space:
            pass
        elif space == 'xspace':
            self.backward()
        elif space == 'kspace':
            self.forward()
        else:
            raise ValueError("space must be either xspace or kspace.")

    def find_mode(self, mode, exact=False):
        # representations.py:247-288
        dk = 2 * np.pi / swap_indices(self.length)
        test = np.ones(tuple(self.local_shape['kspace']), dtype=bool)
        for name, kn in self.k.items():
            i = self.ktrans[name]
            if exact:
                itest = (kn == mode[i])
            else:
                itest = ((kn <= mode[i] + dk[i] / 2.) & (kn > mode[i] - dk[i] / 2.))
            test = test * itest
        index = list(zip(*test.nonzero()))
        if len(index) == 0:
            return None
        elif len(index) == 1:
            return index[0]
        raise ValueError("Multiple modes tested true. This shouldn't happen.")

    def set_fft(self, method):
        self._allocate_memory(method)
        self.fft = self.fwd_np
        self.ifft = self.rev_np

    def fwd_np(self):
        # representations.py:327-329: divide first, rfftn, transpose axes 0<->1
        tr = [1, 0, 2][:self.ndim]
        if FFT_WORKERS > 1:
            import scipy.fft as spfft
            self.kdata[:] = np.transpose(spfft.rfftn(self.xdata / self.global_shape['xspace'].prod(),
                                                     workers=FFT_WORKERS), tr)
            return
        self.kdata[:] = np.transpose(npfft.rfftn(self.xdata / self.global_shape['xspace'].prod()), tr)

    def rev_np(self):
        # representations.py:331-333
        tr = [1, 0, 2][:self.ndim]
        if FFT_WORKERS > 1:
            import scipy.fft as spfft
            self.xdata[:] = spfft.irfftn(np.transpose(self.kdata, tr), s=tuple(self.global_shape['xspace']),
                                         workers=FFT_WORKERS) * self.global_shape['xspace'].prod()
            return
        self.xdata[:] = npfft.irfftn(np.transpose(self.kdata, tr)) * self.global_shape['xspace'].prod()

    def forward(self):
        # representations.py:335-345
        if self._curr_space == 'kspace':
            raise ValueError("Forward transform cannot be called from kspace.")
        self.fft()
        self.data = self.kdata
        self._curr_space = 'kspace'
        self.dealias()
        self.fwd_count += 1

    def backward(self):
        # representations.py:347-357
        if self._curr_space == 'xspace':
            raise ValueError("Backward transform cannot be called from xspace.")
        self.dealias()
        self.ifft()
        self.data = self.xdata
        self._curr_space = 'xspace'
        self.rev_count += 1

    def set_dealiasing(self, dealiasing):
        # representations.py:359-382
        if dealiasing == '2/3':
            self.dealias = self.dealias_23
        elif dealiasing == '2/3 cython':
            self.dealias = self.dealias_23_cython
        elif dealiasing == '2/3 spherical':
            self.dealias = self.dealias_23_spherical
        elif dealiasing in ['None', None, 0]:
            self.dealias = self.zero_nyquist
        else:
            raise NotImplementedError("Specified dealiasing method not implemented.")

    def dealias_23(self):
        # representations.py:384-397
        if self.ndim == 2:
            dmask = ((np.abs(self.k['x']) >= 2. / 3. * self.kny[0]) |
                     (np.abs(self.k['y']) >= 2. / 3. * self.kny[1]))
        else:
            dmask = ((np.abs(self.k['x']) >= 2. / 3. * self.kny[2]) |
                     (np.abs(self.k['y']) >= 2. / 3. * self.kny[0]) |
                     (np.abs(self.k['z']) >= 2. / 3. * self.kny[1]))
        self.require_space('kspace')
        self.data[np.broadcast_to(dmask, self.data.shape)] = 0.

    def dealias_23_cython(self):
        # representations.py:399-408 -> dealias_cy_{2d,3d}.dealias_23
        self.require_space('kspace')
        if self.ndim == 2:
            _cstage.dealias_23(self.data, self.k['x'], self.k['y'], self.kny)
        else:
            _cstage.dealias_23(self.data, self.k['x'], self.k['y'], self.k['z'], self.kny)

    def dealias_23_spherical(self):
        dmask = (np.sqrt(self.k2()) >= 2 / 3. * np.min(self.kny))
        self.require_space('kspace')
        self.data[dmask] = 0.

    def deriv(self, dim):
        # representations.py:419-425
        self.require_space('kspace')
        np.multiply(self.data, 1j * self.k[dim], self.deriv_data)
        return self.deriv_data

    def k2(self, no_zero=False, set_zero=1.):
        # representations.py:427-440
        k2 = np.zeros(tuple(self.local_shape['kspace']))
        for k in self.k.values():
            k2 += k ** 2
        if no_zero:
            k2[k2 == 0] = set_zero
        return k2

    def zero_nyquist(self):
        # representations.py:442-455
        if self.ndim == 2:
            dmask = ((np.abs(self.k['x']) == self.kny[0]) |
                     (np.abs(self.k['y']) == self.kny[1]))
        else:
            dmask = ((np.abs(self.k['x']) == self.kny[2]) |
                     (np.abs(self.k['y']) == self.kny[0]) |
                     (np.abs(self.k['z']) == self.kny[1]))
        self.require_space('kspace')
        self.data[np.broadcast_to(dmask, self.data.shape)] = 0.

    def xspace_grid(self, open=False):
        refgrid = np.ogrid if open else np.mgrid
        grid = refgrid[tuple(slice(int(i)) for i in self.local_shape['xspace'])]
        grid = [g.astype(np.float64) for g in grid]
        grid[0] += self.offset['xspace']
        dx = self.dx()
        for i in range(self.ndim):
            grid[i] *= dx[i]
        return grid

    def dx(self):
        return self.length / self.global_shape['xspace']


class FourierShearRepresentation(FourierRepresentation):
    """representations.py:558-740: shearing-box component.

    k['y'] is a full-shape array that follows the shear (``_update_k``,
    627-643).  The transforms follow the FFTW branch (``fwd_fftw`` /
    ``rev_fftw``, 676-704): x transform, phase shift exp(+-i S kx y t) of the
    x-transformed rows, y/z transforms, forward normalised by 1/N, backward
    unnormalised.  The reference's numpy branch (``rev_np``, 721-737) ends by
    scaling ``kdata`` instead of ``xdata`` by N, so its backward transform
    comes out divided by N; the oracle does not restate that slip.  The 2/3
    rule is the Cython kernel's sheared-ky branch (dealias_cy_3d.pyx:39-45,
    dealias_cy_2d.pyx:36-40), written here in numpy."""

    _static_k = False

    def __init__(self, sd, shape, length):
        FourierRepresentation.__init__(self, sd, shape, length)
        # representations.py:596-617
        self._ky = self.k['y'].copy()
        self.k['y'] = self.k['y'] * np.ones_like(self.k['x'])
        ksize = self.global_shape['kspace'][self.ktrans['x']]
        xsize = self.global_shape['xspace'][self.xtrans['x']]
        xkx = npfft.fftfreq(xsize)[:ksize] * 2. * self.kny[self.ktrans['x']]
        if xsize % 2 == 0:
            xkx[-1] *= -1.
        xkx = xkx.reshape((self.ndim - 1) * (1,) + (ksize,))
        y = self.xspace_grid(open=True)[self.xtrans['y']]
        self._phase_rate = self.sd.parameters['shear_rate'] * xkx * y
        self._wave_rate = self.sd.parameters['shear_rate'] * self.k['x']
        self._update_k()

    def _update_k(self):
        # representations.py:627-643
        np.subtract(self._ky, self._wave_rate * self.sd.time, self.k['y'])
        kny_y = self.kny[3 - self.ndim]
        if self.k['y'].min() <= -kny_y:
            self.k['y'][self.k['y'] <= -kny_y] += 2 * kny_y
        if self.k['y'].max() > kny_y:
            self.k['y'][self.k['y'] > kny_y] -= 2 * kny_y
        self.dealias()

    def _sheared_mask(self):
        if self.ndim == 2:
            tx, ty = 2. / 3. * self.kny[0], 2. / 3. * self.kny[1]
            return (((self.k['x'] >= tx) | (self.k['x'] <= -tx)) |
                    ((self.k['y'] >= ty) | (self.k['y'] <= -ty)))
        tx, ty, tz = 2. / 3. * self.kny[2], 2. / 3. * self.kny[0], 2. / 3. * self.kny[1]
        return (((self.k['x'] >= tx) | (self.k['x'] <= -tx)) |
                ((self.k['y'] >= ty) | (self.k['y'] <= -ty)) |
                ((self.k['z'] >= tz) | (self.k['z'] <= -tz)))

    def dealias_23(self):
        self.require_space('kspace')
        self.data[np.broadcast_to(self._sheared_mask(), self.data.shape)] = 0.

    dealias_23_cython = dealias_23

    def set_dealiasing(self, dealiasing):
        if dealiasing not in ('2/3', '2/3 cython'):
            raise NotImplementedError("the oracle's shearing box restates the 2/3 rules only")
        self.dealias = self.dealias_23

    def fwd_np(self):
        # representations.py:676-691 (fwd_fftw)
        m = npfft.rfft(self.xdata, axis=-1)
        m = m * np.exp(1j * self._phase_rate * self.sd.time)
        tr = [1, 0, 2][:self.ndim]
        k = np.transpose(m, tr)
        if self.ndim == 2:
            k = npfft.fft(k, axis=1)
        else:
            k = npfft.fftn(k, axes=(0, 1))
        self.kdata[:] = k / self.global_shape['xspace'].prod()

    def rev_np(self):
        # representations.py:693-704 (rev_fftw: unnormalised inverse)
        gx = self.global_shape['xspace']
        if self.ndim == 2:
            k = npfft.ifft(self.kdata, axis=1) * gx[0]
        else:
            k = npfft.ifftn(self.kdata, axes=(0, 1)) * (gx[0] * gx[1])
        tr = [1, 0, 2][:self.ndim]
        m = np.transpose(k, tr)
        m = m * np.exp(-1j * self._phase_rate * self.sd.time)
        self.xdata[:] = npfft.irfft(m, n=int(gx[-1]), axis=-1) * gx[-1]
