"""Device diagnostics against the oracle's restatement of the reference's
volume averages and power spectrum (volume_average.py, analysis_set.py:778-815).
Tolerance: 1e-12 relative (compensated FP64 sums vs numpy pairwise sums)."""
import numpy as np
import pytest

from oracle import diagnostics as OD, physics as OP
from oracle.representation import FourierRepresentation as OracleRep


def both(dd, cls, shape, fields, params=None):
    M = dd.mods
    ro = getattr(OP, cls)(shape, OracleRep)
    rg = getattr(M, cls)(shape, M.FourierRepresentation)
    for r in (ro, rg):
        r.parameters.update(params or {})
    do, dg = ro.create_fields(0.), rg.create_fields(0.)
    for (f, c), a in fields.items():
        do[f][c]['kspace'] = a.copy()
        dg[f][c]['kspace'] = a
    return do, dg


def close(a, b, tol=1e-12):
    return abs(a - b) <= tol * max(abs(b), 1e-300)


@pytest.mark.gpu
@pytest.mark.parametrize("shape", [(32, 32, 32), (64, 64, 64)])
def test_3d_volume_averages_and_spectrum(dd, cuda, shape):
    u = dd.init_cond.turbulence_3d(shape, seed=3)
    do, dg = both(dd, 'IncompressibleHydro', shape, {('u', i): u[i] for i in range(3)}, {'nu': 5e-3})
    D = dd.diagnostics
    assert close(D.ekin(dg), OD.ekin(do))
    assert abs(D.ekin(dg) - 1.0) < 1e-12          # the generator's unit energy
    assert close(D.energy_dissipation(dg, 5e-3), OD.energy_dissipation(do, 5e-3))
    assert close(D.divergence_sum(dg), OD.divergence_sum(do), 1e-9) or OD.divergence_sum(do) < 1e-10
    assert D.divergence_l2(dg) < 1e-26           # solenoidal to roundoff
    kg, eg = D.power_spectrum(dg['u'])
    ko, eo = OD.compute_spectrum(do['u'])
    np.testing.assert_allclose(kg, ko, rtol=0, atol=1e-14)
    np.testing.assert_allclose(eg, eo, rtol=1e-12, atol=1e-300)


@pytest.mark.gpu
def test_2d_volume_averages_and_spectrum(dd, cuda):
    shape = (128, 128)
    u = dd.init_cond.turbulence_2d(shape, seed=2)
    do, dg = both(dd, 'IncompressibleHydro', shape, {('u', 0): u[0], ('u', 1): u[1]}, {'nu': 1e-3})
    D = dd.diagnostics
    assert close(D.ekin(dg), OD.ekin(do))
    assert close(D.enstrophy(dg), OD.enstrophy(do))
    kg, eg = D.power_spectrum(dg['u'])
    ko, eo = OD.compute_spectrum(do['u'])
    np.testing.assert_allclose(eg, eo, rtol=1e-12, atol=1e-300)


@pytest.mark.gpu
def test_mhd_magnetic_energy_and_helicity(dd, cuda):
    shape = (32, 32, 32)
    u = dd.init_cond.turbulence_3d(shape, seed=4)
    b = dd.init_cond.turbulence_3d(shape, seed=5, energy_target=0.5)
    f = {('u', i): u[i] for i in range(3)}
    f.update({('B', i): b[i] for i in range(3)})
    do, dg = both(dd, 'IncompressibleMHD', shape, f)
    D = dd.diagnostics
    assert close(D.emag(dg), OD.ekin(do, 'B'))
    assert abs(D.emag(dg) - 0.5) < 1e-12
    # helicity <u . w> from x-space fields on the host
    M = dd.mods
    uk = [dg['u'][i].to_numpy('kspace') for i in range(3)]
    k = dg['u'][0].k_host
    w = [1j * k['y'] * uk[2] - 1j * k['z'] * uk[1], 1j * k['z'] * uk[0] - 1j * k['x'] * uk[2],
         1j * k['x'] * uk[1] - 1j * k['y'] * uk[0]]
    tr = [1, 0, 2]
    ux = [np.fft.irfftn(np.transpose(c, tr)) * np.prod(shape) for c in uk]
    wx = [np.fft.irfftn(np.transpose(c, tr)) * np.prod(shape) for c in w]
    h = float(np.mean(sum(a * c for a, c in zip(ux, wx))))
    assert abs(D.helicity(dg) - h) < 1e-12 * max(1.0, abs(h))
