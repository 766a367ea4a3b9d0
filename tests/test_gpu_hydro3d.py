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
@pytest.mark.parametrize("shape", [(64, 64, 64), (16, 32, 256)])
def test_fp32_path_error(dd, cuda, shape):
    """FP32 transforms (divergence form for this solenoidal state) against the
    FP64 oracle; (16, 32, 256) runs the FP32 256-point x-pass schedule of the
    headline's FP32 arm."""
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


@pytest.mark.gpu
@pytest.mark.parametrize("shape", [(32, 32, 32), (16, 32, 64), (256, 256, 256)])
def test_divergence_form_step_matches_oracle_and_rotational(dd, cuda, shape):
    """A solenoidal state takes the divergence form (physics 2: 3 + 5
    transforms per RHS); its RK4 step equals the oracle's and the rotational
    form's to 1e-12 relative L2."""
    u0 = dd.init_cond.turbulence_3d(shape, seed=7)
    rg, dg = gpu_hydro(dd, shape, 5e-3, u0)
    dd.mods.RK4(rg).do_advance(dg, 2e-3)
    assert rg.last_phys3d == 2
    rr, dr = gpu_hydro(dd, shape, 5e-3, u0)
    rr.nonlinear_form = 'rotational'
    dd.mods.RK4(rr).do_advance(dr, 2e-3)
    assert rr.last_phys3d == 0
    assert rel_l2(host_u(dg), host_u(dr)) < 1e-12
    if shape[0] <= 64:
        ro, do = oracle_hydro(shape, 5e-3, u0)
        OT.RK4(ro).do_advance(do, 2e-3)
        ref = [do['u'][i]['kspace'] for i in range(3)]
        assert rel_l2(host_u(dg), ref) < 1e-12


@pytest.mark.gpu
def test_non_solenoidal_state_takes_the_rotational_form(dd, cuda):
    """A state with a divergent part keeps the rotational form (equal to the
    reference's advective form for any state) and matches the oracle."""
    shape = (32, 32, 32)
    rng = np.random.Generator(np.random.PCG64(8))
    u0 = dd.init_cond.turbulence_3d(shape, seed=8)
    kx, ky, kz = dd.kgrid.k_tables(shape, (2 * np.pi,) * 3)
    grad = [kx[None, None, :], ky[:, None, None], kz[None, :, None]]
    phi = np.zeros_like(u0[0])
    phi[1:4, 1:4, 1:4] = rng.normal(size=(3, 3, 3)) * 0.05
    u1 = [u0[i] + 1j * grad[i] * phi for i in range(3)]
    rg, dg = gpu_hydro(dd, shape, 5e-3, u1)
    dd.mods.RK4(rg).do_advance(dg, 2e-3)
    assert rg.last_phys3d == 0
    ro, do = oracle_hydro(shape, 5e-3, u1)
    OT.RK4(ro).do_advance(do, 2e-3)
    assert rel_l2(host_u(dg), [do['u'][i]['kspace'] for i in range(3)]) < 1e-12


@pytest.mark.gpu
@pytest.mark.parametrize("prec", [0, 1])
def test_divergence_form_rhs_matches_rotational(dd, cuda, prec):
    """dd_rhs3d physics 2 against physics 0 on a solenoidal state (FP64 to
    1e-12, FP32 to 1e-5), and dd_divergence_sums against numpy."""
    import ctypes
    import torch
    shape = (32, 32, 32)
    u0 = dd.init_cond.turbulence_3d(shape, seed=9)
    plan = dd.engine.get_plan(shape, (2 * np.pi,) * 3)
    u = [torch.from_numpy(c).cuda() for c in u0]
    up, _a = dd._lib.ptr_array([c.data_ptr() for c in u])
    ik2 = dd.mods.IncompressibleHydro(shape, dd.mods.FourierRepresentation).inv_k2_table(plan)
    outs = []
    for phys in (0, 2):
        n = ctypes.c_size_t()
        dd._lib.call("dd_rhs3d_workspace_size", plan.handle, phys, prec, ctypes.byref(n))
        ws = torch.empty(n.value, dtype=torch.uint8, device="cuda")
        d = [torch.empty_like(c) for c in u]
        dp, _b = dd._lib.ptr_array([c.data_ptr() for c in d])
        dd._lib.call("dd_rhs3d", plan.handle, phys, None, up, dp, dd.engine.dptr(ik2), prec, 1,
                     dd.engine.dptr(ws), ws.numel(), dd.engine.current_stream())
        outs.append([c.cpu().numpy() for c in d])
    assert rel_l2(outs[1], outs[0]) < (1e-12 if prec == 0 else 1e-5)
    sums = torch.empty(2, dtype=torch.float64, device="cuda")
    dd._lib.call("dd_divergence_sums", plan.handle, up, dd.engine.dptr(sums), dd.engine.current_stream())
    kx, ky, kz = dd.kgrid.k_tables(shape, (2 * np.pi,) * 3)
    K = [kx[None, None, :], ky[:, None, None], kz[None, :, None]]
    mx, my, mz = plan.mx, plan.my, plan.mz
    keep = ((np.abs(K[0]) <= mx) & (np.abs(K[1]) <= my) & (np.abs(K[2]) <= mz))
    div = sum(K[i] * u0[i] for i in range(3))
    k2 = K[0] ** 2 + K[1] ** 2 + K[2] ** 2
    ref0 = np.sum(np.abs(div) ** 2 * keep)
    ref1 = np.sum(k2 * sum(np.abs(c) ** 2 for c in u0) * keep)
    got = sums.cpu().numpy()
    assert abs(got[1] - ref1) <= 1e-12 * ref1
    assert got[0] <= 1e-24 * ref1 and ref0 <= 1e-24 * ref1


@pytest.mark.gpu
def test_state_form_is_rechecked_when_the_state_changes(dd, cuda):
    """The fused step reuses its solenoidality / non-kept check while the
    state is only advanced by fused steps, and re-checks it after a write
    through the public API or a touch() after a direct write: a divergent
    state then takes the rotational form, a state with energy outside the kept
    modes has them decayed, both matching the oracle."""
    shape = (32, 32, 32)
    u0 = dd.init_cond.turbulence_3d(shape, seed=12)
    rg, dg = gpu_hydro(dd, shape, 5e-3, u0)
    ti = dd.mods.RK4(rg)
    ti.do_advance(dg, 2e-3)
    ti.do_advance(dg, 2e-3)
    assert rg.last_phys3d == 2
    # a divergent state written through the API
    kx, ky, kz = dd.kgrid.k_tables(shape, (2 * np.pi,) * 3)
    grad = [kx[None, None, :], ky[:, None, None], kz[None, :, None]]
    phi = np.zeros_like(u0[0])
    phi[1:4, 1:4, 1:4] = 0.05
    u1 = [host_u(dg)[i] + 1j * grad[i] * phi for i in range(3)]
    for i in range(3):
        dg['u'][i]['kspace'] = u1[i]
    ti.do_advance(dg, 2e-3)
    assert rg.last_phys3d == 0
    ro, do = oracle_hydro(shape, 5e-3, u1)
    OT.RK4(ro).do_advance(do, 2e-3)
    assert rel_l2(host_u(dg), [do['u'][i]['kspace'] for i in range(3)]) < 1e-12
    # energy outside the kept modes written directly, announced with touch()
    rng = np.random.default_rng(3)
    u2 = [c + 1e-3 * (rng.standard_normal(c.shape) + 1j * rng.standard_normal(c.shape)) for c in u0]
    for i in range(3):
        import torch
        dg['u'][i].kdata.copy_(torch.from_numpy(u2[i]))
        dg['u'][i].touch()
    ti.do_advance(dg, 2e-3)
    ro2, do2 = oracle_hydro(shape, 5e-3, u2)
    OT.RK4(ro2).do_advance(do2, 2e-3)
    assert rel_l2(host_u(dg), [do2['u'][i]['kspace'] for i in range(3)]) < 1e-12
