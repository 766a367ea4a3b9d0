"""RK2trap (time_step.py:312-392; etd1 predictor, etd2rk1 corrector, or euler
with IF None) through the device stage kernels, against the oracle's RK2trap:
<= 1e-12 relative L2 after three steps."""
import numpy as np
import pytest

from oracle import physics as OP, time_step as OT
from oracle.representation import FourierRepresentation as OracleRep


def rel_l2(got, ref):
    num = sum(np.sum(np.abs(g - r) ** 2) for g, r in zip(got, ref))
    den = sum(np.sum(np.abs(r) ** 2) for r in ref)
    return float(np.sqrt(num / den))


def run_pair(dd, cls, shape, params, fields, names, dt, nsteps=3):
    M = dd.mods
    ro = getattr(OP, cls)(shape, OracleRep)
    rg = getattr(M, cls)(shape, M.FourierRepresentation)
    for r in (ro, rg):
        r.parameters.update(params)
    do, dg = ro.create_fields(0.), rg.create_fields(0.)
    for (f, c), a in fields.items():
        do[f][c]['kspace'] = a.copy()
        dg[f][c]['kspace'] = a
    to, tg = OT.RK2trap(ro), M.RK2trap(rg)
    for _ in range(nsteps):
        to.do_advance(do, dt)
        tg.do_advance(dg, dt)
    assert tg.iteration == nsteps and abs(tg.time - nsteps * dt) < 1e-15
    return rel_l2([dg[f][c].to_numpy('kspace') for f, c in names], [do[f][c]['kspace'] for f, c in names])


@pytest.mark.gpu
@pytest.mark.parametrize("nu", [5e-3, 0.0])
def test_rk2trap_hydro3d(dd, cuda, nu):
    shape = (32, 32, 32)
    u = dd.init_cond.turbulence_3d(shape, seed=61)
    names = [('u', 0), ('u', 1), ('u', 2)]
    assert run_pair(dd, 'IncompressibleHydro', shape, {'nu': nu}, {n: u[n[1]] for n in names}, names, 2e-3) < 1e-12


@pytest.mark.gpu
def test_rk2trap_hydro2d(dd, cuda):
    shape = (128, 128)
    u = dd.init_cond.turbulence_2d(shape, seed=62)
    names = [('u', 0), ('u', 1)]
    assert run_pair(dd, 'IncompressibleHydro', shape, {'nu': 1e-3}, {n: u[n[1]] for n in names}, names, 1e-3) < 1e-12


@pytest.mark.gpu
def test_rk2trap_boussinesq2d(dd, cuda):
    shape = (64, 64)
    T = dd.init_cond.band_limited_noise_2d(shape, seed=63)
    u = dd.init_cond.turbulence_2d(shape, seed=64, energy_target=1e-2)
    names = [('u', 0), ('u', 1), ('T', 0)]
    f = {('u', 0): u[0], ('u', 1): u[1], ('T', 0): T}
    p = {'nu': 2e-3, 'kappa': 2e-3, 'g': 1., 'alpha_t': 1., 'beta': 1., 'boussinesq_direction': 'y'}
    assert run_pair(dd, 'BoussinesqHydro', shape, p, f, names, 1e-2) < 1e-12


@pytest.mark.gpu
def test_rk2trap_mhd(dd, cuda):
    shape = (16, 16, 16)
    u = dd.init_cond.turbulence_3d(shape, seed=65, k0=3.0)
    b = dd.init_cond.turbulence_3d(shape, seed=66, k0=3.0)
    names = [('u', 0), ('u', 1), ('u', 2), ('B', 0), ('B', 1), ('B', 2)]
    f = {('u', i): u[i] for i in range(3)}
    f.update({('B', i): b[i] for i in range(3)})
    assert run_pair(dd, 'IncompressibleMHD', shape, {'nu': 5e-3, 'eta': 5e-3}, f, names, 1e-3) < 1e-12
