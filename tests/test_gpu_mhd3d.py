"""3D incompressible MHD against the oracle, the FP32 transform/product path
against FP64, and the linear Alfven-wave known answer of the reference's
sample (samples/incompressible_mhd/alfven_wave/alfven_wave.py:11-54).
FP64 tolerance: relative L2 <= 1e-12 per RHS and per step."""
import numpy as np
import pytest

from oracle import physics as OP, time_step as OT
from oracle.representation import FourierRepresentation as OracleRep

NAMES = [('u', 0), ('u', 1), ('u', 2), ('B', 0), ('B', 1), ('B', 2)]


def rel_l2(got, ref):
    num = sum(np.sum(np.abs(g - r) ** 2) for g, r in zip(got, ref))
    den = sum(np.sum(np.abs(r) ** 2) for r in ref)
    return float(np.sqrt(num / den))


def fields(dd, shape, seed):
    u = dd.init_cond.turbulence_3d(shape, seed=seed, k0=3.0)
    b = dd.init_cond.turbulence_3d(shape, seed=seed + 1000, k0=3.0)
    return u + b


def setup(dd, shape, params, comps):
    M = dd.mods
    ro = OP.IncompressibleMHD(shape, OracleRep)
    rg = M.IncompressibleMHD(shape, M.FourierRepresentation)
    for r in (ro, rg):
        r.parameters.update(params)
    do, dg = ro.create_fields(0.), rg.create_fields(0.)
    for (f, c), a in zip(NAMES, comps):
        do[f][c]['kspace'] = a.copy()
        dg[f][c]['kspace'] = a
    return ro, do, rg, dg


def host(data, gpu):
    return [data[f][c].to_numpy('kspace') if gpu else data[f][c]['kspace'] for f, c in NAMES]


@pytest.mark.gpu
@pytest.mark.parametrize("shape", [(16, 16, 16), (32, 32, 32), (16, 32, 64)])
@pytest.mark.parametrize("rho0", [1.0, 2.5])
def test_mhd_rhs(dd, cuda, shape, rho0):
    ro, do, rg, dg = setup(dd, shape, {'nu': 5e-3, 'eta': 5e-3, 'rho0': rho0}, fields(dd, shape, 1))
    eo, eg = ro.create_fields(0.), rg.create_fields(0.)
    ro.RHS(do, eo)
    rg.RHS(dg, eg)
    assert rel_l2(host(eg, True), host(eo, False)) < 1e-12


@pytest.mark.gpu
@pytest.mark.parametrize("shape", [(16, 16, 16), (32, 32, 32)])
def test_mhd_rk4_steps(dd, cuda, shape):
    ro, do, rg, dg = setup(dd, shape, {'nu': 5e-3, 'eta': 8e-3}, fields(dd, shape, 2))
    to, tg = OT.RK4(ro), dd.mods.RK4(rg)
    for _ in range(3):
        to.do_advance(do, 1e-3)
        tg.do_advance(dg, 1e-3)
        assert rel_l2(host(dg, True), host(do, False)) < 1e-12


@pytest.mark.gpu
def test_mhd_fp32_per_field_error(dd, cuda):
    shape = (64, 64, 64)
    comps = fields(dd, shape, 3)
    ro, do, rg, dg = setup(dd, shape, {'nu': 5e-3, 'eta': 5e-3}, comps)
    OT.RK4(ro).do_advance(do, 1e-3)
    dd.config.decfg.set('FFT', 'precision', 'fp32')
    try:
        dd.mods.RK4(rg).do_advance(dg, 1e-3)
    finally:
        dd.config.decfg.set('FFT', 'precision', 'fp64')
    g, r = host(dg, True), host(do, False)
    for i in range(6):
        assert rel_l2([g[i]], [r[i]]) < 1e-5, NAMES[i]


@pytest.mark.gpu
def test_alfven_wave_known_answer(dd, cuda):
    """A transverse Alfven wave on a uniform B0 is an exact nonlinear
    solution of ideal MHD: each Fourier amplitude rotates as exp(-i w t),
    w = vA k.B0/|B0|, vA = |B0| / sqrt(4 pi rho0)."""
    shape = (32, 32, 32)
    M = dd.mods
    rhs = M.IncompressibleMHD(shape, M.FourierRepresentation)
    data = rhs.create_fields(0.)
    k = np.array([3., 2., 1.])                    # (z, y, x), as in the sample
    B0 = np.array([1., 0., 0.])                   # (z, y, x): along z
    u1 = 1e-3 * np.array([0., -1., 2.]) / np.sqrt(5)
    vA = np.sqrt(1.0 / (4 * np.pi))
    omega = vA * np.dot(k, B0)
    B1 = -np.dot(k, B0) * u1 / omega
    ksim = dd.kgrid.swap_indices(list(k))
    rep = data['B']['y']
    idx, idxm = rep.find_mode(ksim), rep.find_mode([-v for v in ksim])
    comp = {'z': 0, 'y': 1, 'x': 2}
    hostB = {c: np.zeros(rep.kdata.shape, complex) for c in 'xyz'}
    hostU = {c: np.zeros(rep.kdata.shape, complex) for c in 'xyz'}
    hostB['z'][0, 0, 0] = B0[0]
    for ix in (idx, idxm):
        if ix is None:
            continue
        for c in 'xyz':
            hostB[c][ix] += B1[comp[c]] / 2.
            hostU[c][ix] += u1[comp[c]] / 2.
    for c in 'xyz':
        data['B'][c]['kspace'] = hostB[c]
        data['u'][c]['kspace'] = hostU[c]
    ti = M.RK4(rhs)
    dt, nsteps = 0.01, 186
    for _ in range(nsteps):
        ti.do_advance(data, dt)
    t = dt * nsteps
    phase = np.exp(-1j * omega * t)
    for c in 'xy':
        got = data['u'][c].to_numpy('kspace')[idx]
        want = hostU[c][idx] * phase
        assert abs(got - want) < 1e-6 * abs(hostU[c][idx]) + 1e-14, (c, got, want)
        gotb = data['B'][c].to_numpy('kspace')[idx]
        assert abs(gotb - hostB[c][idx] * phase) < 1e-6 * abs(hostB[c][idx]) + 1e-14


@pytest.mark.gpu
@pytest.mark.parametrize("shape,rho0", [((32, 32, 32), 1.0), ((16, 32, 64), 2.5), ((256, 256, 256), 1.0)])
def test_mhd_divergence_form_step(dd, cuda, shape, rho0):
    """Solenoidal u and B take the divergence form (physics 3: 6 + 8
    transforms per RHS); two RK4 steps equal the curl form's and the oracle's
    to 1e-12 relative L2."""
    params = {'nu': 5e-3, 'eta': 5e-3, 'rho0': rho0}
    comps = fields(dd, shape, 5)
    M = dd.mods
    runs = []
    for form in ('auto', 'rotational'):
        rg = M.IncompressibleMHD(shape, M.FourierRepresentation)
        rg.parameters.update(params)
        rg.nonlinear_form = form
        dg = rg.create_fields(0.)
        for (f, c), a in zip(NAMES, comps):
            dg[f][c]['kspace'] = a
        ti = M.RK4(rg)
        for _ in range(2):
            ti.do_advance(dg, 1e-3)
        runs.append((rg.last_phys3d, host(dg, True)))
    assert runs[0][0] == 3 and runs[1][0] == 1
    assert rel_l2(runs[0][1], runs[1][1]) < 1e-12
    if shape[0] <= 64:
        ro, do, _rg, _dg = setup(dd, shape, params, comps)
        to = OT.RK4(ro)
        for _ in range(2):
            to.do_advance(do, 1e-3)
        assert rel_l2(runs[0][1], host(do, False)) < 1e-12


@pytest.mark.gpu
def test_mhd_divergent_field_takes_the_curl_form(dd, cuda):
    """A magnetic field with a divergent part keeps the curl forms (which the
    reference computes for any field) and matches the oracle."""
    shape = (32, 32, 32)
    comps = fields(dd, shape, 6)
    kx, ky, kz = dd.kgrid.k_tables(shape, (2 * np.pi,) * 3)
    grad = [kx[None, None, :], ky[:, None, None], kz[None, :, None]]
    phi = np.zeros_like(comps[0])
    phi[1:3, 1:3, 1:3] = 0.05
    comps = comps[:3] + [comps[3 + i] + 1j * grad[i] * phi for i in range(3)]
    params = {'nu': 5e-3, 'eta': 5e-3, 'rho0': 1.0}
    ro, do, rg, dg = setup(dd, shape, params, comps)
    dd.mods.RK4(rg).do_advance(dg, 1e-3)
    OT.RK4(ro).do_advance(do, 1e-3)
    assert rg.last_phys3d == 1
    assert rel_l2(host(dg, True), host(do, False)) < 1e-12
