"""3D incompressible hydro parity against the oracle (the reference's
physics/time-stepping restated on numpy + the reference's Cython kernels).

Tolerance (FP64): relative L2 over all components <= 1e-12 per RHS and per
step, the bar the reference's own CPU path is held to.  The FP32
transform/product path is reported against FP64 with a 1e-5 bound."""
import numpy as np
import pytest

from oracle import physics as OP, time_step as OT
from oracle.representation import FourierRepresentation as OracleRep


def rel_l2(got, ref):
    num = sum(np.sum(np.abs(g - r) ** 2) for g, r in zip(got, ref))
    den = sum(np.sum(np.abs(r) ** 2) for r in ref)
    return float(np.sqrt(num / den))


def oracle_hydro(shape, nu, u0):
    rhs = OP.IncompressibleHydro(shape, OracleRep)
    rhs.parameters['nu'] = nu
    data = rhs.create_fields(0.)
    for i in range(3):
        data['u'][i]['kspace'] = u0[i].copy()
    return rhs, data


def gpu_hydro(dd, shape, nu, u0):
    M = dd.mods
    rhs = M.IncompressibleHydro(shape, M.FourierRepresentation)
    rhs.parameters['nu'] = nu
    data = rhs.create_fields(0.)
    for i in range(3):
        data['u'][i]['kspace'] = u0[i]
    return rhs, data


def host_u(data):
    return [data['u'][i].to_numpy('kspace') for i in range(3)]


SHAPES = [(16, 16, 16), (32, 32, 32), (16, 32, 64), (64, 64, 64)]


@pytest.mark.gpu
@pytest.mark.parametrize("shape", SHAPES)
def test_rhs_matches_oracle(dd, cuda, shape):
    u0 = dd.init_cond.turbulence_3d(shape, seed=1)
    ro, do = oracle_hydro(shape, 5e-3, u0)
    dero = ro.create_fields(0.)
    ro.RHS(do, dero)
    rg, dg = gpu_hydro(dd, shape, 5e-3, u0)
    derg = rg.create_fields(0.)
    rg.RHS(dg, derg)
    err = rel_l2(host_u(derg), [dero['u'][i]['kspace'] for i in range(3)])
    assert err < 1e-12, err
    # integrating factors set on the first call, as physics.py:504-513
    IF = derg['u'][0].integrating_factor.cpu().numpy()
    np.testing.assert_array_equal(IF, dero['u'][0].integrating_factor)


@pytest.mark.gpu
@pytest.mark.parametrize("shape", SHAPES)
@pytest.mark.parametrize("nu,dt", [(5e-3, 2e-3), (0.5, 2e-3), (0.0, 1e-3)])
def test_rk4_step_matches_oracle(dd, cuda, shape, nu, dt):
    u0 = dd.init_cond.turbulence_3d(shape, seed=2)
    ro, do = oracle_hydro(shape, nu, u0)
    OT.RK4(ro).do_advance(do, dt)
    rg, dg = gpu_hydro(dd, shape, nu, u0)
    ti = dd.mods.RK4(rg)
    ti.do_advance(dg, dt)
    err = rel_l2(host_u(dg), [do['u'][i]['kspace'] for i in range(3)])
    assert err < 1e-12, err
    assert ti.iteration == 1 and abs(ti.time - dt) < 1e-15


@pytest.mark.gpu
def test_rk4_generic_path_and_multistep(dd, cuda):
    shape = (32, 32, 32)
    u0 = dd.init_cond.turbulence_3d(shape, seed=3)
    ro, do = oracle_hydro(shape, 5e-3, u0)
    to = OT.RK4(ro)
    rg, dg = gpu_hydro(dd, shape, 5e-3, u0)
    tg = dd.mods.RK4(rg)
    rg2, dg2 = gpu_hydro(dd, shape, 5e-3, u0)
    tg2 = dd.mods.RK4(rg2)
    tg2.use_fused = False
    for step in range(10):
        to.do_advance(do, 2e-3)
        tg.do_advance(dg, 2e-3)
        tg2.do_advance(dg2, 2e-3)
        ref = [do['u'][i]['kspace'] for i in range(3)]
        assert rel_l2(host_u(dg), ref) < 1e-12 * (step + 1)
        assert rel_l2(host_u(dg2), ref) < 1e-12 * (step + 1)


@pytest.mark.gpu
def test_rk2mid_generic_path(dd, cuda):
    shape = (32, 16, 32)
    u0 = dd.init_cond.turbulence_3d(shape, seed=4)
    ro, do = oracle_hydro(shape, 5e-3, u0)
    to = OT.RK2mid(ro)
    rg, dg = gpu_hydro(dd, shape, 5e-3, u0)
    tg = dd.mods.RK2mid(rg)
    for _ in range(3):
        to.do_advance(do, 2e-3)
        tg.do_advance(dg, 2e-3)
    assert rel_l2(host_u(dg), [do['u'][i]['kspace'] for i in range(3)]) < 1e-12


@pytest.mark.gpu
def test_non_dealiased_state_decays_like_reference(dd, cuda):
    """Energy outside the kept modes is never forced and decays by the
    integrating factor (etd1 with zero derivative), as in the reference."""
    shape = (16, 16, 16)
    rng = np.random.default_rng(7)
    u0 = dd.init_cond.turbulence_3d(shape, seed=5)
    noisy = [c + 1e-3 * (rng.standard_normal(c.shape) + 1j * rng.standard_normal(c.shape)) for c in u0]
    ro, do = oracle_hydro(shape, 0.05, noisy)
    OT.RK4(ro).do_advance(do, 0.01)
    rg, dg = gpu_hydro(dd, shape, 0.05, noisy)
    dd.mods.RK4(rg).do_advance(dg, 0.01)
    assert rel_l2(host_u(dg), [do['u'][i]['kspace'] for i in range(3)]) < 1e-12


@pytest.mark.gpu
def test_fp32_path_error(dd, cuda):
    shape = (64, 64, 64)
    u0 = dd.init_cond.turbulence_3d(shape, seed=6)
    ro, do = oracle_hydro(shape, 5e-3, u0)
    OT.RK4(ro).do_advance(do, 2e-3)
    dd.config.decfg.set('FFT', 'precision', 'fp32')
    try:
        rg, dg = gpu_hydro(dd, shape, 5e-3, u0)
        dd.mods.RK4(rg).do_advance(dg, 2e-3)
    finally:
        dd.config.decfg.set('FFT', 'precision', 'fp64')
    err = rel_l2(host_u(dg), [do['u'][i]['kspace'] for i in range(3)])
    assert err < 1e-5, err


@pytest.mark.gpu
@pytest.mark.parametrize("shape", [(16, 16, 16), (32, 32, 32), (64, 64, 64)])
def test_df64_rhs_and_rk4_match_oracle(dd, cuda, shape):
    """Double-float transform arithmetic (FP32 pipes, ~48-bit significands)
    meets the FP64 bar: <= 1e-12 relative L2 per RHS and per step."""
    u0 = dd.init_cond.turbulence_3d(shape, seed=7)
    ro, do = oracle_hydro(shape, 5e-3, u0)
    dero = ro.create_fields(0.)
    ro.RHS(do, dero)
    ref_rhs = [dero['u'][i]['kspace'].copy() for i in range(3)]
    ro2, do2 = oracle_hydro(shape, 5e-3, u0)
    OT.RK4(ro2).do_advance(do2, 2e-3)
    dd.config.decfg.set('FFT', 'precision', 'df64')
    try:
        rg, dg = gpu_hydro(dd, shape, 5e-3, u0)
        derg = rg.create_fields(0.)
        rg.RHS(dg, derg)
        e_rhs = rel_l2(host_u(derg), ref_rhs)
        rg2, dg2 = gpu_hydro(dd, shape, 5e-3, u0)
        dd.mods.RK4(rg2).do_advance(dg2, 2e-3)
        e_step = rel_l2(host_u(dg2), [do2['u'][i]['kspace'] for i in range(3)])
    finally:
        dd.config.decfg.set('FFT', 'precision', 'fp64')
    assert e_rhs < 1e-12, e_rhs
    assert e_step < 1e-12, e_step


@pytest.mark.gpu
def test_df64_not_offered_for_2d(dd, cuda):
    shape = (32, 32)
    M = dd.mods
    rhs = M.IncompressibleHydro(shape, M.FourierRepresentation)
    data = rhs.create_fields(0.)
    for i, c in enumerate(dd.init_cond.turbulence_2d(shape, seed=1)):
        data['u'][i]['kspace'] = c
    dd.config.decfg.set('FFT', 'precision', 'df64')
    try:
        with pytest.raises(NotImplementedError):
            rhs.RHS(data, rhs.create_fields(0.))
    finally:
        dd.config.decfg.set('FFT', 'precision', 'fp64')


@pytest.mark.gpu
def test_rk4_step_matches_oracle_at_256(dd, cuda):
    """The headline configuration itself: one fused RK4 step at 256^3
    (nu = 5e-3, dt = 2e-3) against the oracle, <= 1e-12 relative L2."""
    shape = (256, 256, 256)
    u0 = dd.init_cond.turbulence_3d(shape, seed=0)
    ro, do = oracle_hydro(shape, 5e-3, u0)
    OT.RK4(ro).do_advance(do, 2e-3)
    rg, dg = gpu_hydro(dd, shape, 5e-3, u0)
    dd.mods.RK4(rg).do_advance(dg, 2e-3)
    err = rel_l2(host_u(dg), [do['u'][i]['kspace'] for i in range(3)])
    assert err < 1e-12, err
