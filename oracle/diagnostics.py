"""CPU oracle -- test infrastructure only.

Restatement of the reference's k-space diagnostics
(dedalus/analysis/volume_average.py:71-118, 180-200, 254-295) and of
PowerSpectrum._compute_spectrum (dedalus/analysis/analysis_set.py:778-815)
on the oracle's representation objects.
"""
import numpy as np


def volume_average(values, kx_axis):
    """volume_average.py:86-96 (single process)."""
    if kx_axis == 2:
        return 2 * values[..., 1:].sum() + values[..., 0].sum()
    return 2 * values[1:, ...].sum() + values[0, ...].sum()


def _kx_axis(comp):
    return comp.ktrans['x']


def ekin(data, name='u'):
    f = data[name]
    s = sum(0.5 * np.abs(c['kspace']) ** 2 for i, c in f)
    return float(volume_average(s, _kx_axis(f[0])).real)


def energy_dissipation(data, nu):
    u = data['u']
    s = 0.5 * ((np.abs(u['z'].deriv('y').copy() - u['y'].deriv('z'))) ** 2
               + (np.abs(u['x'].deriv('z').copy() - u['z'].deriv('x'))) ** 2
               + (np.abs(u['y'].deriv('x').copy() - u['x'].deriv('y'))) ** 2)
    return float(volume_average(2 * nu * s, _kx_axis(u[0])).real)


def enstrophy(data):
    u = data['u']
    s = 0.5 * np.abs((u['y'].deriv('x').copy() - u['x'].deriv('y')) ** 2)
    return float(volume_average(s, _kx_axis(u[0])).real)


def divergence_sum(data, name='u'):
    f = data[name]
    div = 0
    for i, c in f:
        div = div + c.deriv(f.ctrans[i]).copy()
    return float(np.abs(div).sum())


def compute_spectrum(field, norm=1.):
    """analysis_set.py:778-815."""
    kmag = np.sqrt(field[0].k2())
    power = np.zeros_like(kmag)
    for cindex, comp in field:
        power += np.abs(comp['kspace']) ** 2
    if field.ndim == 2:
        power1d = norm * power * 2. * np.pi * kmag
    else:
        power1d = norm * power * 4. * np.pi * kmag ** 2
    kmax = np.sqrt(np.sum(field[0].kny ** 2))
    n = np.min(field[0].global_shape['xspace']) / 2.
    n = int(np.min([n, 100]))
    kbottom = np.linspace(0, kmax, n, endpoint=False)
    ktop = kbottom + kbottom[1]
    spectrum = np.zeros_like(kbottom)
    cnt = np.zeros_like(kbottom)
    for i in range(kbottom.size):
        mask = (kmag >= kbottom[i]) & (kmag < ktop[i]) & (power1d != 0)
        spectrum[i] = np.sum(power1d[mask])
        cnt[i] = float(np.sum(mask))
    cnt[cnt == 0] = 1.
    return kbottom + kbottom[1] / 2., spectrum / cnt
