"""CFL time step against the oracle: ``compute_dt`` / ``set_dtlist`` of the
three physics (dedalus/physics/physics.py:151-158, 601-610, 714-721,
830-836), ``max_square`` of a vector field (dedalus/data_objects/fields.py:
153-157, here one device reduction, dd_max_square) and the integrator's
5% growth cap (dedalus/time_stepping/time_step.py:170-179).

Tolerance: the squares of the grid values are exact and their maximum is
order-independent, so the only difference from the oracle is the inverse
transform's rounding (<= 1e-13 relative); dt is compared to 1e-12
relative.  As in the reference, reading max_square leaves every component of
the field in grid space, and a step taken afterwards still matches the
oracle to 1e-12."""
import ctypes

import numpy as np
import pytest

from oracle import physics as OP, time_step as OT
from oracle.representation import FourierRepresentation as OracleRep


def rel_l2(got, ref):
    num = sum(np.sum(np.abs(g - r) ** 2) for g, r in zip(got, ref))
    den = sum(np.sum(np.abs(r) ** 2) for r in ref)
    return float(np.sqrt(num / den))


BPAR = {'nu': 2e-3, 'kappa': 2e-3, 'g': 1., 'alpha_t': 1., 'beta': 1., 'boussinesq_direction': 'y'}


def case(dd, kind):
    """(class name, shape, parameters, {(field, comp): k array}) per physics."""
    if kind == 'hydro3d':
        shape = (32, 32, 32)
        u = dd.init_cond.turbulence_3d(shape, seed=21)
        return 'IncompressibleHydro', shape, {'nu': 5e-3}, {('u', i): u[i] for i in range(3)}
    if kind == 'hydro2d':
        shape = (64, 64)
        u = dd.init_cond.turbulence_2d(shape, seed=22)
        return 'IncompressibleHydro', shape, {'nu': 1e-3}, {('u', i): u[i] for i in range(2)}
    if kind == 'bouss2d':
        shape = (64, 64)
        T = dd.init_cond.band_limited_noise_2d(shape, seed=23)
        # |u|max > N = 1, so the advective limit is the smaller one and a
        # halved state doubles it (the buoyancy-wave limit dx/N is fixed)
        u = dd.init_cond.turbulence_2d(shape, seed=24, energy_target=20.0)
        return 'BoussinesqHydro', shape, BPAR, {('u', 0): u[0], ('u', 1): u[1], ('T', 0): T}
    shape = (32, 32, 32)
    u = dd.init_cond.turbulence_3d(shape, seed=25, k0=3.0)
    b = dd.init_cond.turbulence_3d(shape, seed=26, k0=3.0, energy_target=4.0)
    f = {('u', i): u[i] for i in range(3)}
    f.update({('B', i): b[i] for i in range(3)})
    return 'IncompressibleMHD', shape, {'nu': 5e-3, 'eta': 5e-3, 'rho0': 1.5}, f


def setup(dd, kind, CFL):
    name, shape, params, fields = case(dd, kind)
    M = dd.mods
    ro = getattr(OP, name)(shape, OracleRep)
    rg = getattr(M, name)(shape, M.FourierRepresentation)
    for r in (ro, rg):
        r.parameters.update(params)
    do, dg = ro.create_fields(0.), rg.create_fields(0.)
    for (f, c), a in fields.items():
        do[f][c]['kspace'] = a.copy()
        dg[f][c]['kspace'] = a
    return ro, do, OT.RK2mid(ro, CFL=CFL), rg, dg, M.RK2mid(rg, CFL=CFL), list(fields)


KINDS = ['hydro3d', 'hydro2d', 'bouss2d', 'mhd3d']


@pytest.mark.gpu
@pytest.mark.parametrize("kind", KINDS)
def test_compute_dt_matches_oracle(dd, cuda, kind):
    ro, do, to, rg, dg, tg, names = setup(dd, kind, 0.3)
    dto, dtg = ro.compute_dt(do), rg.compute_dt(dg)
    assert abs(dtg - dto) <= 1e-12 * dto, (dtg, dto)
    assert len(rg.dtlist) == len(ro.dtlist) == {'hydro3d': 1, 'hydro2d': 1, 'bouss2d': 2, 'mhd3d': 2}[kind]
    for a, b in zip(rg.dtlist, ro.dtlist):
        assert abs(a - b) <= 1e-12 * b
    # max_square leaves the velocity components in grid space, as the reference's c['xspace'] does
    for i in range(rg.ndim):
        assert dg['u'][i]._curr_space == 'xspace' and do['u'][i]._curr_space == 'xspace'
    # a step from there (the state transforms back lazily) still matches the oracle
    to.do_advance(do, dto)
    tg.do_advance(dg, dto)
    got = [dg[f][c].to_numpy('kspace') for f, c in names]
    ref = [do[f][c]['kspace'] for f, c in names]
    assert rel_l2(got, ref) < 1e-12


@pytest.mark.gpu
@pytest.mark.parametrize("kind", ['hydro3d', 'bouss2d', 'mhd3d'])
def test_cfl_dt_growth_cap_matches_oracle(dd, cuda, kind):
    """Three CFL steps; before the second the state is halved on both sides,
    so the new CFL dt would double and the 5% cap sets it to 1.05 dt_old."""
    ro, do, to, rg, dg, tg, names = setup(dd, kind, 0.2)
    seq_o, seq_g = [], []
    for step in range(3):
        if step == 1:
            for f, c in names:
                a = do[f][c]['kspace'] * 0.5
                do[f][c]['kspace'] = a
                dg[f][c]['kspace'] = a
        dto, dtg = to.cfl_dt(do), tg.cfl_dt(dg)
        seq_o.append(dto)
        seq_g.append(dtg)
        to.do_advance(do, dto)
        tg.do_advance(dg, dto)
    np.testing.assert_allclose(seq_g, seq_o, rtol=1e-12, atol=0)
    assert seq_g[1] == 1.05 * seq_g[0] and seq_o[1] == 1.05 * seq_o[0]
    assert abs(tg.dt_old - to.dt_old) <= 1e-12 * to.dt_old
    got = [dg[f][c].to_numpy('kspace') for f, c in names]
    ref = [do[f][c]['kspace'] for f, c in names]
    assert rel_l2(got, ref) < 1e-12


@pytest.mark.gpu
def test_max_square_kernel_edge_cases(dd, cuda):
    """dd_max_square through the C ABI: empty input, one component, several
    components of ragged content, a NaN anywhere, and negative values."""
    import torch
    lib = dd._lib
    st = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    out = torch.full((), -1.0, dtype=torch.float64, device=cuda)

    def run(arrs, n=None):
        ts = [torch.from_numpy(np.ascontiguousarray(a, dtype=np.float64)).to(cuda) for a in arrs]
        pp, _k = lib.ptr_array([t.data_ptr() for t in ts])
        lib.call("dd_max_square", len(ts), pp, ts[0].numel() if n is None else n,
                 ctypes.c_void_p(out.data_ptr()), st)
        return float(out.item())

    rng = np.random.default_rng(5)
    assert run([np.zeros(4)], n=0) == 0.0
    a = rng.standard_normal(1000003)
    assert run([a]) == float(np.max(a ** 2))
    comps = [rng.standard_normal(70001) * s for s in (1.0, 3.0, 0.5)]
    comps[2][12345] = -17.25
    assert run(comps) == max(float(np.max(c ** 2)) for c in comps) == 17.25 ** 2
    comps[1][7] = np.nan
    assert np.isnan(run(comps))
    with pytest.raises(ValueError):
        lib.call("dd_max_square", 0, None, 10, ctypes.c_void_p(out.data_ptr()), st)
