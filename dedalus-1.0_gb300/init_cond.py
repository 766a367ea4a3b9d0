"""Seeded synthetic initial conditions for the benchmark configurations.

The reference's generators (dedalus/init_cond/init_cond.py:281-341 turb_new,
391-408 MIT_vortices) draw from numpy's global legacy RNG; these use
``numpy.random.Generator(PCG64(seed))`` and build every field as the
reference's do: random phases taken from the transform of a real random
field (so the spectrum is Hermitian by construction), a shell amplitude
``sqrt(2 E(k) / (4 pi k^2))`` in 3D (``/(2 pi k)`` in 2D, init_cond.py:298-301),
solenoidal projection (fields.py:169-195), 2/3 dealiasing, and a final
normalisation to the requested kinetic energy E = 1/2 <|u|^2>.

All arrays are host numpy complex128 in the reference k-layout ((ky, kz, kx) in
3D, (kx, ky) in 2D), for any representation or the oracle to load.
"""
import numpy as np

from . import kgrid


def spectrum(k, k0=4.0):
    """E(k) ~ k^4 exp(-2 (k/k0)^2)."""
    return k ** 4 * np.exp(-2.0 * (k / k0) ** 2)


def _forward(x):
    """The reference's forward transform (representations.py:327-329)."""
    tr = [1, 0, 2][:x.ndim]
    return np.transpose(np.fft.rfftn(x / np.prod(x.shape)), tr).copy()


def _grid(xshape, length):
    k, kny, ktrans = kgrid.wavenumbers(xshape, length)
    mx, my, mz = kgrid.kept_bounds(xshape, length, '2/3 cython')
    kshape = kgrid.kspace_shape(list(xshape))
    ndim = len(xshape)
    kv = {n: np.broadcast_to(v, kshape) for n, v in k.items()}
    k2 = np.zeros(kshape)
    for v in k.values():
        k2 = k2 + v ** 2
    # kept mask from the index bounds
    idx = np.indices(kshape)
    if ndim == 3:
        ky_i, kz_i, kx_i = idx
        Ny, Nz = kshape[0], kshape[1]
        kept = (kx_i <= mx) & ((ky_i <= my) | (ky_i >= Ny - my)) & ((kz_i <= mz) | (kz_i >= Nz - mz))
    else:
        kx_i, ky_i = idx
        Ny = kshape[1]
        kept = (kx_i <= mx) & ((ky_i <= my) | (ky_i >= Ny - my))
    return kv, k2, kept, kshape


def volume_average_k(a, kx_axis):
    """Sum of a k-space density with Hermitian weights (volume_average.py:86-96)."""
    if kx_axis == 2:
        return 2 * a[..., 1:].sum() + a[..., 0].sum()
    return 2 * a[1:, ...].sum() + a[0, ...].sum()


def energy(u_hat, ndim):
    """1/2 <|u|^2> from k-space components (volume_average.py:108-118)."""
    e = sum(0.5 * np.abs(c) ** 2 for c in u_hat)
    return float(volume_average_k(e, 2 if ndim == 3 else 0).real)


def _phases(rng, xshape):
    w = _forward(rng.random(xshape))
    a = np.abs(w)
    return np.where(a > 0, w / np.where(a > 0, a, 1.0), 0.0)


def _project(u, kv, k2, ndim):
    """F - k (k.F) / k^2, the solenoidal projection of fields.py:169-195."""
    names = ('x', 'y', 'z')[:ndim]
    kdotu = sum(u[i] * kv[n] for i, n in enumerate(names))
    k2n = np.where(k2 == 0, 1.0, k2)
    return [u[i] - kv[n] * kdotu / k2n for i, n in enumerate(names)]


def turbulence_3d(xshape, length=None, seed=0, k0=4.0, energy_target=1.0):
    """Random-phase solenoidal velocity with E(k) ~ k^4 exp(-2(k/k0)^2)."""
    length = length or (2 * np.pi,) * 3
    rng = np.random.Generator(np.random.PCG64(seed))
    kv, k2, kept, kshape = _grid(xshape, length)
    kk = np.sqrt(k2)
    kk1 = np.where(kk == 0, 1.0, kk)
    amp = np.where(kk == 0, 0.0, np.sqrt(2.0 * spectrum(kk, k0) / (4 * np.pi * kk1 ** 2)))
    u = [amp * _phases(rng, xshape) for _ in range(3)]
    u = _project(u, kv, k2, 3)
    u = [np.where(kept, c, 0.0) for c in u]
    s = np.sqrt(energy_target / energy(u, 3))
    return [np.ascontiguousarray(c * s) for c in u]


def turbulence_2d(xshape, length=None, seed=0, k0=4.0, energy_target=1.0):
    """2D velocity from a random-phase vorticity with E(k) ~ k^4 exp(-2(k/k0)^2):
    w_hat = sqrt(k E(k) / pi) e^(i theta), psi = w / k^2, u = (d_y psi, -d_x psi)
    (init_cond.py:405-408)."""
    length = length or (2 * np.pi,) * 2
    rng = np.random.Generator(np.random.PCG64(seed))
    kv, k2, kept, kshape = _grid(xshape, length)
    kk = np.sqrt(k2)
    w = np.sqrt(kk * spectrum(kk, k0) / np.pi) * _phases(rng, xshape)
    psi = w / np.where(k2 == 0, 1.0, k2)
    u = [psi * (1j * kv['y']), -(psi * (1j * kv['x']))]
    u = [np.where(kept, c, 0.0) for c in u]
    s = np.sqrt(energy_target / energy(u, 2))
    return [np.ascontiguousarray(c * s) for c in u]


def band_limited_noise_2d(xshape, length=None, seed=0, kmax=8.0, amplitude=1e-3):
    """Temperature perturbation: flat-amplitude random phases on 0 < |k| <= kmax,
    scaled to rms amplitude `amplitude` in x-space."""
    length = length or (2 * np.pi,) * 2
    rng = np.random.Generator(np.random.PCG64(seed))
    kv, k2, kept, kshape = _grid(xshape, length)
    t = _phases(rng, xshape) * ((k2 > 0) & (np.sqrt(k2) <= kmax) & kept)
    rms2 = float(volume_average_k(np.abs(t) ** 2, 0).real)
    return np.ascontiguousarray(t * (amplitude / np.sqrt(rms2)))


def load(data, name, comps):
    """Write host k-space arrays into data[name] components (kspace)."""
    for i, c in enumerate(comps):
        data[name][i]['kspace'] = c
