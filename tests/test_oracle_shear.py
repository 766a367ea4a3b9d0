"""Oracle restatement of the shearing-box representation
(representations.py:558-740) and the shear / rotation branches of the physics,
checked on the CPU against known answers:

* a shearing wave cos(kx x + (ky - S kx t) y + kz z) sampled on the grid at
  time t is one k entry, 1/2 at (ky, kz, kx) (the phase shift of the
  transforms undoes the shear exactly);
* k -> x -> k reproduces the sheared-dealiased spectrum; the wavenumbers wrap
  into (-kny, kny];
* a single 2D inviscid shearing vortex wave (an exact nonlinear solution)
  conserves its vorticity k x u in shearing coordinates when the pressure
  solve uses the current k^2, while u itself changes (the transient growth of
  a leading wave); with the reference's cached k^2 it does not.
"""
import numpy as np
import pytest

from oracle import representation as R
from oracle import physics as P
from oracle import time_step as T


def _shear_state(shape, S, t, length=None, fields=(('u', 'VectorField'),)):
    length = length or (2 * np.pi,) * len(shape)
    params = {'shear_rate': S}
    classes = R and __import__('oracle.fields', fromlist=['x']).create_field_classes(
        R.FourierShearRepresentation, shape, length)
    from oracle.fields import StateData
    return StateData(t, shape, length, classes, field_list=list(fields), params=params)


@pytest.mark.parametrize("shape", [(16, 16), (16, 16, 16)])
def test_shearing_wave_is_one_mode(shape):
    S, t = 1.0, 0.3
    kx, ky, kz = 2, 3, 1
    sd = _shear_state(shape, S, t, fields=(('f', 'ScalarField'),))
    c = sd['f'].components[0]
    grid = c.xspace_grid()
    if len(shape) == 2:
        y, x = grid
        f = np.cos(kx * x + (ky - S * kx * t) * y)
    else:
        z, y, x = grid
        f = np.cos(kx * x + (ky - S * kx * t) * y + kz * z)
    c['xspace'] = f
    k = c['kspace']
    idx = (kx, ky) if len(shape) == 2 else (ky, kz, kx)
    assert abs(k[idx] - 0.5) < 1e-14
    k2 = k.copy()
    k2[idx] = 0
    assert np.max(np.abs(k2)) < 1e-14
    # and back
    back = c['xspace']
    assert np.max(np.abs(back - f)) < 1e-13


@pytest.mark.parametrize("shape", [(16, 32), (16, 16, 16)])
def test_roundtrip_reproduces_the_sheared_dealiased_spectrum(shape):
    S, t = 1.5, 0.7
    sd = _shear_state(shape, S, t, fields=(('f', 'ScalarField'),))
    c = sd['f'].components[0]
    rng = np.random.Generator(np.random.PCG64(3))
    c['xspace'] = rng.normal(size=shape)
    k0 = c['kspace'].copy()          # forward applies the sheared 2/3 rule
    c.require_space('xspace')
    k1 = c['kspace']
    assert np.max(np.abs(k1 - k0)) < 1e-14 * np.max(np.abs(k0)) * 10
    # every surviving mode satisfies the sheared rule
    ky = np.broadcast_to(c.k['y'], k0.shape)
    kny_y = c.kny[3 - len(shape)]
    assert np.all(k0[np.abs(ky) >= 2. / 3. * kny_y] == 0)


def test_wavenumbers_wrap_into_the_nyquist_band():
    shape = (16, 16, 16)
    sd = _shear_state(shape, 2.0, 0.0)
    c = sd['u'][0]
    for t in (0.5, 1.7, 3.1):
        sd.set_time(t)
        ky = c.k['y']
        assert ky.shape == (16, 1, 9)
        kny = c.kny[0]
        ref = c._ky - 2.0 * c.k['x'] * t
        ref = np.where(ref <= -kny, ref + 2 * kny, ref)
        ref = np.where(ref > kny, ref - 2 * kny, ref)
        assert np.array_equal(ky, ref)


def _vortex_wave(RHS, data, kx, ky, A):
    c = data['u'][0]
    y, x = c.xspace_grid()
    t = data.time
    kyt = ky - RHS.parameters['shear_rate'] * kx * t
    s = np.sin(kx * x + kyt * y)
    data['u']['x']['xspace'] = -A * kyt * s
    data['u']['y']['xspace'] = A * kx * s


def _vorticity(data, kx, ky):
    ux, uy = data['u']['x']['kspace'], data['u']['y']['kspace']
    kyt = data['u']['x'].k['y'][kx, ky]
    return 1j * (kx * uy[kx, ky] - kyt * ux[kx, ky]), uy[kx, ky]


@pytest.mark.parametrize("laplace_k2,conserved", [("current", True), ("cached", False)])
def test_inviscid_shearing_vortex_wave_conserves_vorticity(laplace_k2, conserved):
    shape = (32, 32)
    S, kx, ky = 1.0, 1, 4           # a leading wave: |k_y(t)| = |4 - t| shrinks, u grows
    RHS = P.IncompressibleHydro(shape, R.FourierShearRepresentation)
    RHS.parameters['shear_rate'] = S
    RHS.laplace_k2 = laplace_k2
    data = RHS.create_fields(0.)
    _vortex_wave(RHS, data, kx, ky, 1e-3)
    w0, u0 = _vorticity(data, kx, ky)
    ti = T.RK4(RHS)
    dt = 1e-2
    for _ in range(300):
        ti.do_advance(data, dt)
    w1, u1 = _vorticity(data, kx, ky)
    if conserved:
        assert abs(u1) > 3 * abs(u0)                # transient growth of u_y (|k|^2: 17 -> 2)
        assert abs(w1 - w0) < 1e-8 * abs(w0), (w0, w1)
    else:
        assert abs(w1 - w0) > 1e-3 * abs(w0), (w0, w1)
