"""2D parity against the oracle: incompressible hydro (the 128^2, nu = 1e-3,
RK2mid, dt = 1e-3 configuration, including its full 100 steps) and
Boussinesq (direction 'y', N^2 = g alpha beta = 1, nu = kappa = 2e-3).
Tolerance: relative L2 over all fields <= 1e-12 (per step)."""
import numpy as np
import pytest

from oracle import physics as OP, time_step as OT
from oracle.representation import FourierRepresentation as OracleRep


def rel_l2(got, ref):
    num = sum(np.sum(np.abs(g - r) ** 2) for g, r in zip(got, ref))
    den = sum(np.sum(np.abs(r) ** 2) for r in ref)
    return float(np.sqrt(num / den))


def setup(dd, cls_name, shape, params, fields):
    M = dd.mods
    ro = getattr(OP, cls_name)(shape, OracleRep)
    rg = getattr(M, cls_name)(shape, M.FourierRepresentation)
    for r in (ro, rg):
        r.parameters.update(params)
    do, dg = ro.create_fields(0.), rg.create_fields(0.)
    for (name, i), arr in fields.items():
        do[name][i]['kspace'] = arr.copy()
        dg[name][i]['kspace'] = arr
    return ro, do, rg, dg


def state(data, names, gpu):
    return [data[f][c].to_numpy('kspace') if gpu else data[f][c]['kspace'] for f, c in names]


HYD = [('u', 0), ('u', 1)]
BOU = [('u', 0), ('u', 1), ('T', 0)]


def hydro_fields(dd, shape, seed):
    u = dd.init_cond.turbulence_2d(shape, seed=seed)
    return {('u', 0): u[0], ('u', 1): u[1]}


def bouss_fields(dd, shape, seed, with_u=True):
    T = dd.init_cond.band_limited_noise_2d(shape, seed=seed)
    u = dd.init_cond.turbulence_2d(shape, seed=seed + 1, energy_target=1e-2)
    if not with_u:
        u = [np.zeros_like(T), np.zeros_like(T)]
    return {('u', 0): u[0], ('u', 1): u[1], ('T', 0): T}


BPAR = {'nu': 2e-3, 'kappa': 2e-3, 'g': 1., 'alpha_t': 1., 'beta': 1., 'boussinesq_direction': 'y'}


@pytest.mark.gpu
@pytest.mark.parametrize("shape", [(32, 32), (128, 128), (64, 256), (512, 512)])
def test_hydro2d_rhs(dd, cuda, shape):
    ro, do, rg, dg = setup(dd, 'IncompressibleHydro', shape, {'nu': 1e-3}, hydro_fields(dd, shape, 1))
    eo, eg = ro.create_fields(0.), rg.create_fields(0.)
    ro.RHS(do, eo)
    rg.RHS(dg, eg)
    assert rel_l2(state(eg, HYD, True), state(eo, HYD, False)) < 1e-12


@pytest.mark.gpu
def test_hydro2d_config1_100_steps(dd, cuda):
    shape = (128, 128)
    ro, do, rg, dg = setup(dd, 'IncompressibleHydro', shape, {'nu': 1e-3}, hydro_fields(dd, shape, 0))
    to, tg = OT.RK2mid(ro), dd.mods.RK2mid(rg)
    worst = 0.
    for step in range(100):
        to.do_advance(do, 1e-3)
        tg.do_advance(dg, 1e-3)
        if step % 10 == 9 or step < 3:
            worst = max(worst, rel_l2(state(dg, HYD, True), state(do, HYD, False)))
    assert worst < 1e-12, worst
    assert tg.iteration == 100 and abs(dg.time - 0.1) < 1e-12


@pytest.mark.gpu
@pytest.mark.parametrize("shape", [(64, 64), (128, 128), (256, 256)])
@pytest.mark.parametrize("with_u", [False, True])
def test_boussinesq2d_rhs(dd, cuda, shape, with_u):
    ro, do, rg, dg = setup(dd, 'BoussinesqHydro', shape, BPAR, bouss_fields(dd, shape, 2, with_u))
    eo, eg = ro.create_fields(0.), rg.create_fields(0.)
    ro.RHS(do, eo)
    rg.RHS(dg, eg)
    assert rel_l2(state(eg, BOU, True), state(eo, BOU, False)) < 1e-12


@pytest.mark.gpu
@pytest.mark.parametrize("shape", [(64, 64), (256, 256)])
def test_boussinesq2d_rk2mid_steps(dd, cuda, shape):
    ro, do, rg, dg = setup(dd, 'BoussinesqHydro', shape, BPAR, bouss_fields(dd, shape, 3))
    to, tg = OT.RK2mid(ro), dd.mods.RK2mid(rg)
    for step in range(5):
        to.do_advance(do, 1e-2)
        tg.do_advance(dg, 1e-2)
        assert rel_l2(state(dg, BOU, True), state(do, BOU, False)) < 1e-12


@pytest.mark.gpu
def test_boussinesq2d_generic_rk2mid_and_rk4(dd, cuda):
    shape = (64, 64)
    ro, do, rg, dg = setup(dd, 'BoussinesqHydro', shape, BPAR, bouss_fields(dd, shape, 4))
    to, tg = OT.RK2mid(ro), dd.mods.RK2mid(rg)
    tg.use_fused = False
    for _ in range(3):
        to.do_advance(do, 1e-2)
        tg.do_advance(dg, 1e-2)
    assert rel_l2(state(dg, BOU, True), state(do, BOU, False)) < 1e-12
    ro, do, rg, dg = setup(dd, 'BoussinesqHydro', shape, BPAR, bouss_fields(dd, shape, 5))
    OT.RK4(ro).do_advance(do, 1e-2)
    dd.mods.RK4(rg).do_advance(dg, 1e-2)
    assert rel_l2(state(dg, BOU, True), state(do, BOU, False)) < 1e-12


@pytest.mark.gpu
def test_boussinesq2d_default_direction_raises_keyerror(dd, cuda):
    """The reference's default direction 'z' has no 2D velocity component."""
    shape = (32, 32)
    M = dd.mods
    rg = M.BoussinesqHydro(shape, M.FourierRepresentation)
    rg.parameters['boussinesq_direction'] = 'z'
    dg = rg.create_fields(0.)
    with pytest.raises(KeyError):
        rg.RHS(dg, rg.create_fields(0.))


@pytest.mark.gpu
def test_gravity_wave_known_answer(dd, cuda):
    """Gravity-wave eigenmode of the reference's sample
    (samples/boussinesq_hydro/gravity_wave/2d_gmode_kx1_kz1.py:36-54), in 2D
    with gravity along y: at k = (1, 1) the amplitudes rotate as exp(-i w t),
    w = beta sqrt(kx^2 / (kx^2 + ky^2)) with N^2 = g alpha beta = 1."""
    shape = (32, 32)
    M = dd.mods
    rhs = M.BoussinesqHydro(shape, M.FourierRepresentation)
    rhs.parameters.update({'g': 1., 'alpha_t': 1., 'beta': 1., 'nu': 0., 'kappa': 0.,
                           'boussinesq_direction': 'y'})
    data = rhs.create_fields(0.)
    kx, ky, uy = 1., 1., 0.5
    omega = np.sqrt(kx ** 2 / (kx ** 2 + ky ** 2)) * rhs.parameters['beta']
    mode = data['u']['y'].find_mode(np.array([kx, ky]))
    init = {('u', 1): uy, ('u', 0): -ky / kx * uy,
            ('T', 0): -1j * rhs.parameters['beta'] / np.sqrt(kx ** 2 / (kx ** 2 + ky ** 2)) * uy}
    for (f, c), v in init.items():
        a = np.zeros(data[f][c].kdata.shape, complex)
        a[mode] = v
        data[f][c]['kspace'] = a
    ti = M.RK2mid(rhs)
    dt, nsteps = 1e-3, 2000
    for _ in range(nsteps):
        ti.do_advance(data, dt)
    phase = np.exp(-1j * omega * dt * nsteps)
    for (f, c), v in init.items():
        got = data[f][c].to_numpy('kspace')[mode]
        assert abs(got - v * phase) < 1e-5 * abs(v), (f, c, got, v * phase)


@pytest.mark.gpu
@pytest.mark.parametrize("cls,shape", [("IncompressibleHydro", (256, 256)), ("BoussinesqHydro", (256, 256)),
                                       ("BoussinesqHydro", (256, 512))])
def test_divergence_form_2d_steps(dd, cuda, cls, shape):
    """On grids of 256^2 points and more a solenoidal u takes the divergence
    form (physics 2 / 3); five RK2mid steps equal the curl form's and the
    oracle's to 1e-12 relative L2."""
    hydro = cls == "IncompressibleHydro"
    names = HYD if hydro else BOU
    params = {'nu': 1e-3} if hydro else BPAR
    fields = hydro_fields(dd, shape, 4) if hydro else bouss_fields(dd, shape, 5)
    ro, do, rg, dg = setup(dd, cls, shape, params, fields)
    _r2, _d2, rc, dc = setup(dd, cls, shape, params, fields)
    rc.nonlinear_form = 'rotational'
    to, tg, tc = OT.RK2mid(ro), dd.mods.RK2mid(rg), dd.mods.RK2mid(rc)
    for _ in range(5):
        to.do_advance(do, 1e-2 if not hydro else 1e-3)
        tg.do_advance(dg, 1e-2 if not hydro else 1e-3)
        tc.do_advance(dc, 1e-2 if not hydro else 1e-3)
    assert rg.last_phys2d == (2 if hydro else 3) and rc.last_phys2d == (0 if hydro else 1)
    assert rel_l2(state(dg, names, True), state(dc, names, True)) < 1e-12
    assert rel_l2(state(dg, names, True), state(do, names, False)) < 1e-12


@pytest.mark.gpu
def test_divergence_sums_2d(dd, cuda):
    import torch
    shape = (64, 128)
    u = dd.init_cond.turbulence_2d(shape, seed=6)
    rng = np.random.Generator(np.random.PCG64(7))
    v = [u[0] + 0.01 * rng.normal(size=u[0].shape), u[1]]        # a divergent copy as run 1
    slab = torch.from_numpy(np.stack([np.stack([u[0], u[1], u[0]]), np.stack([v[0], v[1], v[0]])])).cuda()
    plan = dd.engine.get_plan(shape, (2 * np.pi,) * 2)
    out = torch.empty(2, dtype=torch.float64, device="cuda")
    fs = slab[0, 0].numel()
    for nrun, runs in ((1, [u]), (2, [u, v])):
        dd._lib.call("dd_divergence_sums2d", plan.handle, nrun, dd.engine.dptr(slab[0, 0]), dd.engine.dptr(slab[0, 1]),
                     3 * fs, dd.engine.dptr(out), dd.engine.current_stream())
        kx, ky, _ = dd.kgrid.k_tables(shape, (2 * np.pi,) * 2)
        KX, KY = kx[:, None], ky[None, :]
        keep = (np.abs(KX) <= plan.mx) & ((np.arange(len(ky)) <= plan.my) | (np.arange(len(ky)) >= len(ky) - plan.my))[None, :]
        r0 = sum(np.sum(np.abs(KX * w[0] + KY * w[1]) ** 2 * keep) for w in runs)
        r1 = sum(np.sum((KX ** 2 + KY ** 2) * (np.abs(w[0]) ** 2 + np.abs(w[1]) ** 2) * keep) for w in runs)
        got = out.cpu().numpy()
        assert abs(got[1] - r1) <= 1e-12 * r1
        assert abs(got[0] - r0) <= 1e-12 * r1
    assert got[0] > 1e-6 * got[1]          # the divergent run shows


@pytest.mark.gpu
@pytest.mark.parametrize("cls,shape", [("IncompressibleHydro", (256, 256)), ("BoussinesqHydro", (512, 512))])
def test_fp32_low_storage_2d_steps(dd, cuda, cls, shape):
    """FP32 transforms on a solenoidal state take the low-storage step
    (complex64 products and stage state, float N and projection, FP64 state
    update): five RK2mid steps keep the divergence form (the state stays
    solenoidal to FP32 accuracy) and their increments agree with the oracle's
    to 1e-4 relative L2."""
    hydro = cls == "IncompressibleHydro"
    names = HYD if hydro else BOU
    params = {'nu': 1e-3} if hydro else BPAR
    fields = hydro_fields(dd, shape, 6) if hydro else bouss_fields(dd, shape, 7)
    init = [fields[k].copy() for k in names]
    dd.config.decfg.set('FFT', 'precision', 'fp32')
    try:
        ro, do, rg, dg = setup(dd, cls, shape, params, fields)
        to, tg = OT.RK2mid(ro), dd.mods.RK2mid(rg)
        dt = 1e-3 if hydro else 1e-2
        for _ in range(5):
            to.do_advance(do, dt)
            tg.do_advance(dg, dt)
            assert rg.last_phys2d == (2 if hydro else 3)
    finally:
        dd.config.decfg.set('FFT', 'precision', 'fp64')
    got = [a - b for a, b in zip(state(dg, names, True), init)]
    ref = [a - b for a, b in zip(state(do, names, False), init)]
    assert rel_l2(got, ref) < 1e-4, rel_l2(got, ref)
