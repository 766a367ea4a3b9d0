"""Parity against the oracle away from the configurations' defaults: boxes
whose sides are not 2 pi (non-integer wavenumbers, so the fused steps take
the direct phi-function / 1/k^2 branch instead of the integer-q tables),
anisotropic boxes, and hyperviscosity (viscosity_order = 2, the IF
nu k^(2 vo) of physics.py:504-522).  Tolerance: 1e-12 relative L2 per RHS /
step, as for the default configurations."""
import numpy as np
import pytest

from oracle import physics as OP, time_step as OT
from oracle.representation import FourierRepresentation as OracleRep


def rel_l2(got, ref):
    num = sum(np.sum(np.abs(g - r) ** 2) for g, r in zip(got, ref))
    den = sum(np.sum(np.abs(r) ** 2) for r in ref)
    return float(np.sqrt(num / den))


def pair(dd, cls, shape, length, params, fields):
    M = dd.mods
    ro = getattr(OP, cls)(shape, OracleRep, length=length)
    rg = getattr(M, cls)(shape, M.FourierRepresentation, length=length)
    for r in (ro, rg):
        r.parameters.update(params)
    do, dg = ro.create_fields(0.), rg.create_fields(0.)
    for (f, c), a in fields.items():
        do[f][c]['kspace'] = a.copy()
        dg[f][c]['kspace'] = a
    return ro, do, rg, dg


def states(do, dg, names):
    return [dg[f][c].to_numpy('kspace') for f, c in names], [do[f][c]['kspace'] for f, c in names]


U3 = [('u', 0), ('u', 1), ('u', 2)]


@pytest.mark.gpu
@pytest.mark.parametrize("shape,length", [((16, 32, 64), (1.5, 2 * np.pi, 4.0)),
                                          ((32, 32, 32), (3.0, 3.0, 3.0)),
                                          ((32, 16, 32), (2 * np.pi, np.pi, 4 * np.pi))])
@pytest.mark.parametrize("vo", [1, 2])
def test_hydro3d_rk4_general_box(dd, cuda, shape, length, vo):
    u = dd.init_cond.turbulence_3d(shape, length=length, seed=31)
    nu = 5e-3 if vo == 1 else 1e-4
    ro, do, rg, dg = pair(dd, 'IncompressibleHydro', shape, length, {'nu': nu, 'viscosity_order': vo},
                          {f: u[f[1]] for f in U3})
    eo, eg = ro.create_fields(0.), rg.create_fields(0.)
    ro.RHS(do, eo)
    rg.RHS(dg, eg)
    assert rel_l2(*states(eo, eg, U3)) < 1e-12
    # fresh objects for the step: the reference sets the integrating factors on
    # the first deriv it is given only (physics.py:538-540)
    ro, do, rg, dg = pair(dd, 'IncompressibleHydro', shape, length, {'nu': nu, 'viscosity_order': vo},
                          {f: u[f[1]] for f in U3})
    OT.RK4(ro).do_advance(do, 2e-3)
    dd.mods.RK4(rg).do_advance(dg, 2e-3)
    assert rel_l2(*states(do, dg, U3)) < 1e-12


@pytest.mark.gpu
@pytest.mark.parametrize("vo", [1, 2])
def test_hydro3d_hyperviscous_integer_box(dd, cuda, vo):
    """2 pi box (integer q tables) with viscosity_order 1 and 2, three steps."""
    shape = (32, 32, 32)
    u = dd.init_cond.turbulence_3d(shape, seed=32)
    nu = 5e-3 if vo == 1 else 2e-5
    ro, do, rg, dg = pair(dd, 'IncompressibleHydro', shape, None, {'nu': nu, 'viscosity_order': vo},
                          {f: u[f[1]] for f in U3})
    to, tg = OT.RK4(ro), dd.mods.RK4(rg)
    for _ in range(3):
        to.do_advance(do, 2e-3)
        tg.do_advance(dg, 2e-3)
    assert rel_l2(*states(do, dg, U3)) < 1e-12


@pytest.mark.gpu
def test_mhd_general_box(dd, cuda):
    shape, length = (16, 32, 32), (2.0, 2 * np.pi, 3.0)
    u = dd.init_cond.turbulence_3d(shape, length=length, seed=33, k0=3.0)
    b = dd.init_cond.turbulence_3d(shape, length=length, seed=34, k0=3.0, energy_target=0.5)
    f = {('u', i): u[i] for i in range(3)}
    f.update({('B', i): b[i] for i in range(3)})
    ro, do, rg, dg = pair(dd, 'IncompressibleMHD', shape, length, {'nu': 5e-3, 'eta': 3e-3}, f)
    names = U3 + [('B', 0), ('B', 1), ('B', 2)]
    OT.RK4(ro).do_advance(do, 1e-3)
    dd.mods.RK4(rg).do_advance(dg, 1e-3)
    assert rel_l2(*states(do, dg, names)) < 1e-12


@pytest.mark.gpu
@pytest.mark.parametrize("shape,length", [((64, 128), (3.0, 2 * np.pi)), ((128, 64), (2 * np.pi, 10.0))])
def test_hydro2d_rk2mid_general_box(dd, cuda, shape, length):
    u = dd.init_cond.turbulence_2d(shape, length=length, seed=35)
    names = [('u', 0), ('u', 1)]
    ro, do, rg, dg = pair(dd, 'IncompressibleHydro', shape, length, {'nu': 1e-3},
                          {('u', 0): u[0], ('u', 1): u[1]})
    to, tg = OT.RK2mid(ro), dd.mods.RK2mid(rg)
    for _ in range(3):
        to.do_advance(do, 1e-3)
        tg.do_advance(dg, 1e-3)
    assert rel_l2(*states(do, dg, names)) < 1e-12


@pytest.mark.gpu
def test_boussinesq2d_general_box(dd, cuda):
    shape, length = (64, 64), (4.0, 2.5)
    T = dd.init_cond.band_limited_noise_2d(shape, length=length, seed=36)
    u = dd.init_cond.turbulence_2d(shape, length=length, seed=37, energy_target=1e-2)
    names = [('u', 0), ('u', 1), ('T', 0)]
    ro, do, rg, dg = pair(dd, 'BoussinesqHydro', shape, length,
                          {'nu': 2e-3, 'kappa': 1e-3, 'g': 1., 'alpha_t': 2., 'beta': 0.5,
                           'boussinesq_direction': 'y'},
                          {('u', 0): u[0], ('u', 1): u[1], ('T', 0): T})
    to, tg = OT.RK2mid(ro), dd.mods.RK2mid(rg)
    for _ in range(3):
        to.do_advance(do, 1e-2)
        tg.do_advance(dg, 1e-2)
    assert rel_l2(*states(do, dg, names)) < 1e-12


@pytest.mark.gpu
@pytest.mark.parametrize("shape", [(512, 32, 32), (32, 512, 32), (32, 32, 512)])
def test_hydro3d_rk4_512_axis(dd, cuda, shape):
    """Length-512 transforms along each axis of the fused 3D step (the largest
    supported length), one RK4 step against the oracle."""
    u = dd.init_cond.turbulence_3d(shape, seed=38)
    ro, do, rg, dg = pair(dd, 'IncompressibleHydro', shape, None, {'nu': 5e-3}, {f: u[f[1]] for f in U3})
    OT.RK4(ro).do_advance(do, 2e-3)
    dd.mods.RK4(rg).do_advance(dg, 2e-3)
    assert rel_l2(*states(do, dg, U3)) < 1e-12


@pytest.mark.gpu
def test_mhd_rk4_512_x_axis(dd, cuda):
    shape = (16, 32, 512)
    u = dd.init_cond.turbulence_3d(shape, seed=39, k0=3.0)
    b = dd.init_cond.turbulence_3d(shape, seed=40, k0=3.0)
    f = {('u', i): u[i] for i in range(3)}
    f.update({('B', i): b[i] for i in range(3)})
    ro, do, rg, dg = pair(dd, 'IncompressibleMHD', shape, None, {'nu': 5e-3, 'eta': 5e-3}, f)
    names = U3 + [('B', 0), ('B', 1), ('B', 2)]
    OT.RK4(ro).do_advance(do, 1e-3)
    dd.mods.RK4(rg).do_advance(dg, 1e-3)
    assert rel_l2(*states(do, dg, names)) < 1e-12


@pytest.mark.gpu
@pytest.mark.parametrize("shape", [(8, 16, 16), (16, 16, 1024)])
def test_3d_lengths_outside_the_supported_range_raise(dd, cuda, shape):
    """8 points (below the fused passes' 16) and 1024 (above the plans' 512)
    raise NotImplementedError, as the reference does for unsupported options."""
    u = dd.init_cond.turbulence_3d(shape, seed=41)
    M = dd.mods
    with pytest.raises(NotImplementedError):
        rg = M.IncompressibleHydro(shape, M.FourierRepresentation)
        rg.parameters['nu'] = 5e-3
        dg = rg.create_fields(0.)
        for i in range(3):
            dg['u'][i]['kspace'] = u[i]
        M.RK4(rg).do_advance(dg, 2e-3)


# ------------------------------------------------ 3 x 2^k lengths (radix-3 pass)
@pytest.mark.gpu
@pytest.mark.parametrize("shape", [(48, 48, 48), (24, 96, 48), (192, 24, 16)])
def test_fft_roundtrip_3x2k(dd, cuda, shape):
    """r2c against numpy's rfftn (the oracle's transform) and c2r back."""
    import torch
    from oracle import closure as OC
    rng = np.random.Generator(np.random.PCG64(50))
    x = rng.normal(size=shape)
    plan = dd.engine.get_plan(shape, (2 * np.pi,) * 3)
    xt = torch.from_numpy(x).cuda()
    k = torch.empty(tuple(plan.kshape), dtype=torch.complex128, device="cuda")
    plan.r2c([xt], [k])
    ref = OC.to_k(x)
    got = k.cpu().numpy()
    assert np.max(np.abs(got - ref)) <= 1e-14 * np.max(np.abs(ref))
    xb = torch.empty_like(xt)
    plan.c2r([k], [xb])
    assert np.max(np.abs(xb.cpu().numpy() - OC.to_x(ref, shape))) <= 1e-12 * np.max(np.abs(x))


@pytest.mark.gpu
@pytest.mark.parametrize("shape", [(48, 48, 48), (24, 96, 48), (16, 192, 32)])
def test_hydro3d_rk4_3x2k(dd, cuda, shape):
    u = dd.init_cond.turbulence_3d(shape, seed=51)
    ro, do, rg, dg = pair(dd, 'IncompressibleHydro', shape, None, {'nu': 5e-3}, {f: u[f[1]] for f in U3})
    OT.RK4(ro).do_advance(do, 2e-3)
    dd.mods.RK4(rg).do_advance(dg, 2e-3)
    assert rel_l2(*states(do, dg, U3)) < 1e-12


@pytest.mark.gpu
def test_mhd_rk4_3x2k(dd, cuda):
    shape = (48, 48, 48)
    u = dd.init_cond.turbulence_3d(shape, seed=52, k0=3.0)
    b = dd.init_cond.turbulence_3d(shape, seed=53, k0=3.0)
    f = {('u', i): u[i] for i in range(3)}
    f.update({('B', i): b[i] for i in range(3)})
    ro, do, rg, dg = pair(dd, 'IncompressibleMHD', shape, None, {'nu': 5e-3, 'eta': 5e-3}, f)
    names = U3 + [('B', 0), ('B', 1), ('B', 2)]
    OT.RK4(ro).do_advance(do, 1e-3)
    dd.mods.RK4(rg).do_advance(dg, 1e-3)
    assert rel_l2(*states(do, dg, names)) < 1e-12


@pytest.mark.gpu
@pytest.mark.parametrize("shape", [(96, 192), (48, 48)])
def test_2d_rk2mid_3x2k(dd, cuda, shape):
    T = dd.init_cond.band_limited_noise_2d(shape, seed=54)
    u = dd.init_cond.turbulence_2d(shape, seed=55, energy_target=1e-2)
    names = [('u', 0), ('u', 1), ('T', 0)]
    ro, do, rg, dg = pair(dd, 'BoussinesqHydro', shape, None,
                          {'nu': 2e-3, 'kappa': 2e-3, 'boussinesq_direction': 'y'},
                          {('u', 0): u[0], ('u', 1): u[1], ('T', 0): T})
    to, tg = OT.RK2mid(ro), dd.mods.RK2mid(rg)
    for _ in range(3):
        to.do_advance(do, 1e-2)
        tg.do_advance(dg, 1e-2)
    assert rel_l2(*states(do, dg, names)) < 1e-12
