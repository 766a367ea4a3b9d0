"""GPU Fourier representation: the drop-in for the reference's
``FourierRepresentation`` (dedalus/data_objects/representations.py:57-557).

Same constructor, shapes, k-layout ((ky, kz, kx) in 3D, (kx, ky) in 2D),
wavenumbers (with the Nyquist sign flip), lazy x/k space switch, forward
normalisation (1/N) and 2/3 dealiasing on both forward and backward
transforms.  ``data['kspace']`` / ``data['xspace']`` return torch CUDA tensors
(complex128 / float64) that alias the component's fixed buffers, as the
reference's arrays alias its FFTW buffers; ``to_numpy(space)`` gives a host
copy.  Transforms and derivatives run in the CUDA library; there is no CPU
path.

Selected by config ``FFT.method = cuda`` (the only method this package
implements; ``numpy`` and ``fftw`` raise NotImplementedError like an unknown
method does in the reference, representations.py:309-310).
"""
import numpy as np
import numpy.fft as npfft
import torch

from . import _lib
from .config import decfg
from .engine import get_plan, current_stream, dptr
from . import kgrid


class Representation:
    def __init__(self, sd, shape, length):
        pass


class FourierRepresentation(Representation):
    """Field component on a periodic Fourier basis, stored on the GPU."""

    _static_k = True

    def __init__(self, sd, shape, length):
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
        self.set_fft(method, dealiasing)
        self._setup_k()
        self._curr_space = 'kspace'
        self.data = self.kdata
        self.fwd_count = 0
        self.rev_count = 0
        # bumped by every public read or write of the data (a read hands out a
        # writable view); the fused steps re-check a state whose version moved
        self._version = 0

    # ------------------------------------------------------------ storage
    def set_fft(self, method, dealiasing):
        if method != 'cuda':
            raise NotImplementedError("Specified FFT method not implemented.")
        if dealiasing not in ('2/3', '2/3 cython', 'None', None, 0):
            raise NotImplementedError("Specified dealiasing method not implemented.")
        self.dealiasing = dealiasing
        self.plan = get_plan(tuple(self.global_shape['xspace']), tuple(self.length), dealiasing)
        self.device = self.plan.device
        ks = kgrid.kspace_shape(list(self.global_shape['xspace']))
        self.global_shape['kspace'] = np.array(ks)
        self.local_shape = {'kspace': self.global_shape['kspace'].copy(),
                            'xspace': self.global_shape['xspace'].copy()}
        self.offset = {'xspace': 0, 'kspace': 0}
        self.kdata = torch.zeros(ks, dtype=torch.complex128, device=self.device)
        self._xdata = None
        self._deriv_data = None
        self.fft = self.fwd_cuda
        self.ifft = self.rev_cuda

    @property
    def xdata(self):
        if self._xdata is None:
            self._xdata = torch.zeros(tuple(self.global_shape['xspace']), dtype=torch.float64, device=self.device)
        return self._xdata

    @property
    def deriv_data(self):
        if self._deriv_data is None:
            self._deriv_data = torch.zeros_like(self.kdata)
        return self._deriv_data

    def _setup_k(self):
        # representations.py:204-233
        k, kny, _ = kgrid.wavenumbers(self.global_shape['xspace'], self.length)
        self.dk = np.asarray(kgrid.swap_indices(2 * np.pi / self.length), dtype=np.float64)
        self.kny = kny
        self.k_host = k
        self.k = {name: torch.from_numpy(np.ascontiguousarray(v)).to(self.device) for name, v in k.items()}

    # ------------------------------------------------------- space access
    def __getitem__(self, space):
        self.require_space(space)
        self._version += 1
        return self.data

    def touch(self):
        """Mark the data as changed: call after writing .kdata / .xdata
        directly (not through ['kspace'] / ['xspace']), so that the fused steps
        re-check the state's form (solenoidal, energy outside the kept modes)."""
        self._version += 1

    def __setitem__(self, space, data):
        # representations.py:144-166
        if space == 'xspace':
            self.data = self.xdata
        elif space == 'kspace':
            self.data = self.kdata
        else:
            raise KeyError("space must be either xspace or kspace.")
        if type(data) == float or type(data) == complex or type(data) == int:
            self.data.fill_(data)
        else:
            if not torch.is_tensor(data):
                data = torch.as_tensor(np.asarray(data))
            sli = tuple(slice(i) for i in self.data.shape)
            src = data[sli]
            if src.shape != self.data.shape:
                src = src.expand(self.data.shape)
            self.data.copy_(src)
        self._curr_space = space
        self._version += 1

    def to_numpy(self, space=None):
        """Host copy of the data in `space` (current space if None)."""
        if space is not None:
            self.require_space(space)
        return self.data.detach().cpu().numpy()

    def require_space(self, space):
        if self._curr_space == space:
            pass
        elif space == 'xspace':
            self.backward()
        elif space == 'kspace':
            self.forward()
        else:
            raise ValueError("space must be either xspace or kspace.")

    # --------------------------------------------------------- transforms
    def fwd_cuda(self):
        self.plan.r2c([self.xdata], [self.kdata])

    def rev_cuda(self):
        self.plan.c2r([self.kdata], [self.xdata])

    def forward(self):
        # representations.py:335-345; r2c already applies 1/N and the dealias mask
        if self._curr_space == 'kspace':
            raise ValueError("Forward transform cannot be called from kspace.")
        self.fft()
        self.data = self.kdata
        self._curr_space = 'kspace'
        self.fwd_count += 1
        self._version += 1

    def backward(self):
        # representations.py:347-357
        if self._curr_space == 'xspace':
            raise ValueError("Backward transform cannot be called from xspace.")
        self.dealias()
        self.ifft()
        self.data = self.xdata
        self._curr_space = 'xspace'
        self.rev_count += 1
        self._version += 1

    def dealias(self):
        """2/3 rule (or Nyquist-only for dealiasing None), in place in k-space."""
        self.require_space('kspace')
        self.plan.dealias(self.kdata)

    dealias_23 = dealias
    dealias_23_cython = dealias

    def zero_nyquist(self):
        # representations.py:442-455
        self.require_space('kspace')
        kx, ky, kz = self.k_host['x'], self.k_host['y'], self.k_host.get('z')
        if self.ndim == 2:
            m = (np.abs(kx) == self.kny[0]) | (np.abs(ky) == self.kny[1])
        else:
            m = (np.abs(kx) == self.kny[2]) | (np.abs(ky) == self.kny[0]) | (np.abs(kz) == self.kny[1])
        mask = torch.from_numpy(np.broadcast_to(m, self.kdata.shape).copy()).to(self.device)
        self.kdata.masked_fill_(mask, 0)

    def deriv(self, dim):
        """i k_dim * data in k-space (representations.py:419-425)."""
        self.require_space('kspace')
        axis = {'x': 0, 'y': 1, 'z': 2}[dim]
        _lib.call("dd_deriv", self.plan.handle, axis, dptr(self.kdata), dptr(self.deriv_data), current_stream())
        return self.deriv_data

    def k2(self, no_zero=False, set_zero=1.):
        """|k|^2 on the k grid (representations.py:427-440), as a device tensor."""
        k2 = np.zeros(tuple(self.local_shape['kspace']))
        for k in self.k_host.values():
            k2 += k ** 2
        if no_zero:
            k2[k2 == 0] = set_zero
        return torch.from_numpy(k2).to(self.device)

    def find_mode(self, mode, exact=False):
        # representations.py:247-288
        dk = 2 * np.pi / kgrid.swap_indices(self.length)
        test = np.ones(tuple(self.local_shape['kspace']), dtype=bool)
        for name, kn in self.k_host.items():
            i = self.ktrans[name]
            if exact:
                itest = (kn == mode[i])
            else:
                itest = ((kn <= mode[i] + dk[i] / 2.) & (kn > mode[i] - dk[i] / 2.))
            test = test * itest
        index = list(zip(*test.nonzero()))
        if len(index) == 0:
            return None
        if len(index) == 1:
            return index[0]
        raise ValueError("Multiple modes tested true. This shouldn't happen.")

    def zero_under_eps(self):
        self.require_space('kspace')
        self.kdata.masked_fill_(self.kdata.abs() < self._eps['kspace'], 0)

    def xspace_grid(self, open=False):
        refgrid = np.ogrid if open else np.mgrid
        grid = refgrid[tuple(slice(int(i)) for i in self.local_shape['xspace'])]
        grid = [g.astype(np.float64) for g in grid]
        dx = self.dx()
        for i in range(self.ndim):
            grid[i] *= dx[i]
        return grid

    def dx(self):
        return self.length / self.global_shape['xspace']


class FourierShearRepresentation(FourierRepresentation):
    """Shearing-box component (representations.py:558-740): k['y'] is a
    full-shape array that follows the shear, k_y(t) = k_y(0) - S k_x t
    wrapped into (-kny, kny], and the transforms multiply the x-transformed
    rows by exp(+-i S k_x y t) between the x and the y/z transforms.  The time
    is that of the component's StateData.  FP64 transforms, '2/3' rules only."""

    _static_k = False

    def __init__(self, sd, shape, length):
        FourierRepresentation.__init__(self, sd, shape, length)
        if self.dealiasing not in ('2/3', '2/3 cython'):
            raise NotImplementedError("the shearing box supports the 2/3 dealiasing rules only")
        if decfg.get('FFT', 'precision', fallback='fp64') != 'fp64':
            raise NotImplementedError("the shearing-box transforms run in FP64")
        # representations.py:596-617
        self._ky = self.k_host['y'].copy()
        self.k_host['y'] = self.k_host['y'] * np.ones_like(self.k_host['x'])
        ksize = self.global_shape['kspace'][self.ktrans['x']]
        xsize = self.global_shape['xspace'][self.xtrans['x']]
        xkx = npfft.fftfreq(xsize)[:ksize] * 2. * self.kny[self.ktrans['x']]
        if xsize % 2 == 0:
            xkx[-1] *= -1.
        xkx = xkx.reshape((self.ndim - 1) * (1,) + (ksize,))
        y = self.xspace_grid(open=True)[self.xtrans['y']]
        self._phase_rate = self.sd.parameters['shear_rate'] * xkx * y
        self._wave_rate = self.sd.parameters['shear_rate'] * self.k_host['x']
        ny = int(self.global_shape['xspace'][self.xtrans['y']])
        self._pr = torch.from_numpy(np.array(self._phase_rate, dtype=np.float64).reshape(ny, ksize)).to(self.device)
        self._kny_y = float(self.kny[3 - self.ndim])
        self._cut = 2. / 3. * self._kny_y
        self._update_k()

    def _update_k(self):
        """representations.py:627-643: shift, wrap, upload, dealias."""
        ky = self.k_host['y']
        np.subtract(self._ky, self._wave_rate * self.sd.time, ky)
        kny_y = self._kny_y
        if ky.min() <= -kny_y:
            ky[ky <= -kny_y] += 2 * kny_y
        if ky.max() > kny_y:
            ky[ky > kny_y] -= 2 * kny_y
        self._kys = torch.from_numpy(np.ascontiguousarray(ky.reshape(-1))).to(self.device)
        self.k['y'] = self._kys.view(ky.shape)
        self.dealias()

    def fwd_cuda(self):
        self.plan.shear_r2c([self.xdata], [self.kdata], self._kys, self._cut, self._pr, self.sd.time)

    def rev_cuda(self):
        self.plan.shear_c2r([self.kdata], [self.xdata], self._kys, self._cut, self._pr, self.sd.time)

    def dealias(self):
        """2/3 rule with the sheared k_y (dealias_cy_{2d,3d}.pyx, full-shape ky branch)."""
        self.require_space('kspace')
        self.plan.shear_dealias([self.kdata], self._kys, self._cut)

    dealias_23 = dealias
    dealias_23_cython = dealias

    def deriv(self, dim):
        if dim != 'y':
            return FourierRepresentation.deriv(self, dim)
        self.require_space('kspace')
        _lib.call("dd_shear_deriv_y", self.plan.handle, dptr(self._kys), dptr(self.kdata), dptr(self.deriv_data),
                  current_stream())
        return self.deriv_data


GpuFourierRepresentation = FourierRepresentation
GpuFourierShearRepresentation = FourierShearRepresentation
