"""Shearing box, rotation, 3D Boussinesq and 2D MHD on the GPU (the
reference-ordered right-hand sides of generic.py over the shearing-box
transforms of csrc/shear.cu) against the CPU oracle.

Tolerances (FP64): transforms 1e-13 of the largest entry; one RHS 1e-12
relative L2 per field (the FFT algorithms differ; every other operation is
rounded as the reference's numpy expressions); integrator steps 1e-11 relative
L2 after the last step.
"""
import numpy as np
import pytest

from oracle import physics as OP
from oracle import representation as OR
from oracle import time_step as OT


def _rel(a, b):
    return float(np.linalg.norm(np.asarray(a) - b) / max(np.linalg.norm(b), 1e-300))


def _states(dd, name, shape, params, t0, shear=True, seed=0, amp=1.0):
    """GPU and oracle physics of class `name` with the same parameters and the
    same initial spectra (an oracle forward transform of random grid values at
    time t0, so that both start dealiased by the rule of that time)."""
    Rg = dd.mods.FourierShearRepresentation if shear else dd.mods.FourierRepresentation
    Ro = OR.FourierShearRepresentation if shear else OR.FourierRepresentation
    G = getattr(dd.mods, name)(shape, Rg)
    O = getattr(OP, name)(shape, Ro)
    for P in (G, O):
        P.parameters.update(params)
    dg, do = G.create_fields(t0), O.create_fields(t0)
    rng = np.random.Generator(np.random.PCG64(seed))
    for f, field in do:
        for i, c in field:
            c['xspace'] = amp * rng.normal(size=shape)
            dg[f][i]['kspace'] = c['kspace'].copy()
    return G, O, dg, do


def _compare(dg, do, tol):
    for f, field in do:
        for i, c in field:
            a = dg[f][i].to_numpy('kspace')
            b = c['kspace']
            assert _rel(a, b) < tol, (f, i, _rel(a, b))


@pytest.mark.gpu
@pytest.mark.parametrize("shape", [(16, 32), (32, 16), (16, 16, 16), (16, 32, 24)])
def test_shear_transforms_match_oracle(dd, cuda, shape):
    S, t = 1.3, 0.9
    G, O, dg, do = _states(dd, "IncompressibleHydro", shape, {"shear_rate": S}, t, seed=1)
    cg, co = dg['u'][0], do['u'][0]
    # forward: same grid values in, same spectrum out
    rng = np.random.Generator(np.random.PCG64(2))
    x = rng.normal(size=shape)
    cg['xspace'] = x
    co['xspace'] = x
    kg, ko = cg.to_numpy('kspace'), co['kspace']
    assert np.max(np.abs(kg - ko)) <= 1e-13 * np.max(np.abs(ko))
    # backward of the same spectrum
    xg, xo = cg.to_numpy('xspace'), co['xspace']
    assert np.max(np.abs(xg - xo)) <= 1e-13 * np.max(np.abs(xo))
    # the sheared wavenumbers are the oracle's
    assert np.array_equal(cg.k_host['y'], co.k['y'])


@pytest.mark.gpu
@pytest.mark.parametrize("shape", [(16, 16), (16, 16, 16)])
def test_shearing_wave_is_one_mode_on_the_gpu(dd, cuda, shape):
    S, t = 1.0, 0.3
    kx, ky, kz = 2, 3, 1
    G = dd.mods.IncompressibleHydro(shape, dd.mods.FourierShearRepresentation)
    G.parameters['shear_rate'] = S
    d = G.create_fields(t)
    c = d['u'][0]
    grid = c.xspace_grid()
    if len(shape) == 2:
        y, x = grid
        f = np.cos(kx * x + (ky - S * kx * t) * y)
    else:
        z, y, x = grid
        f = np.cos(kx * x + (ky - S * kx * t) * y + kz * z)
    c['xspace'] = f
    k = c.to_numpy('kspace')
    idx = (kx, ky) if len(shape) == 2 else (ky, kz, kx)
    assert abs(k[idx] - 0.5) < 1e-14
    k[idx] = 0
    assert np.max(np.abs(k)) < 1e-14


_CASES = [
    ("IncompressibleHydro", (32, 32), {"shear_rate": 1.0, "nu": 1e-2}, True),
    ("IncompressibleHydro", (16, 16, 16), {"shear_rate": 1.5, "nu": 1e-2}, True),
    ("IncompressibleHydro", (16, 16, 16), {"shear_rate": 1.5, "nu": 1e-2, "Omega": np.array([1.0, 0.0, 0.0])},
     True),
    ("IncompressibleHydro", (16, 16, 16), {"nu": 1e-2, "Omega": np.array([0.7, -0.2, 0.3])}, False),
    ("IncompressibleHydro", (32, 32), {"nu": 1e-2, "Omega": 0.8}, False),
    ("BoussinesqHydro", (32, 32), {"shear_rate": 1.0, "nu": 2e-3, "kappa": 2e-3,
                                   "boussinesq_direction": "y"}, True),
    ("BoussinesqHydro", (16, 16, 16), {"nu": 2e-3, "kappa": 2e-3, "boussinesq_direction": "z"}, False),
    ("IncompressibleMHD", (16, 16, 16), {"shear_rate": 1.0, "nu": 5e-3, "eta": 5e-3}, True),
    ("IncompressibleMHD", (32, 32), {"nu": 5e-3, "eta": 5e-3}, False),
    ("IncompressibleMHD", (32, 32), {"shear_rate": 0.8, "nu": 5e-3, "eta": 5e-3}, True),
    ("BoussinesqHydro", (16, 16, 16), {"shear_rate": 1.2, "nu": 2e-3, "kappa": 2e-3, "Omega": np.array([1.0, 0.0, 0.0]),
                                       "boussinesq_direction": "z"}, True),
]


@pytest.mark.gpu
@pytest.mark.parametrize("name,shape,params,shear", _CASES)
def test_rhs_matches_oracle(dd, cuda, name, shape, params, shear):
    t0 = 0.4
    G, O, dg, do = _states(dd, name, shape, params, t0, shear=shear, seed=3)
    kg, ko = G.create_fields(t0), O.create_fields(t0)
    G.RHS(dg, kg)
    O.RHS(do, ko)
    _compare(kg, ko, 1e-12)
    # the integrating factors follow the sheared k^2
    for f, field in ko:
        for i, c in field:
            a, b = kg[f][i].integrating_factor, c.integrating_factor
            if b is None:
                assert a is None
            else:
                assert np.max(np.abs(a.cpu().numpy() - b)) <= 1e-15 * np.max(np.abs(b))


@pytest.mark.gpu
@pytest.mark.parametrize("integrator", ["RK2mid", "RK2trap", "RK4"])
@pytest.mark.parametrize("case", [0, 1, 5, 7])
def test_steps_match_oracle(dd, cuda, integrator, case):
    name, shape, params, shear = _CASES[case]
    t0 = 0.1
    G, O, dg, do = _states(dd, name, shape, params, t0, shear=shear, seed=4, amp=0.3)
    tg, to = getattr(dd.mods, integrator)(G), getattr(OT, integrator)(O)
    for _ in range(4):
        tg.do_advance(dg, 5e-3)
        to.do_advance(do, 5e-3)
    assert abs(dg.time - do.time) < 1e-15
    _compare(dg, do, 1e-11)


@pytest.mark.gpu
def test_shearing_vortex_wave_conserves_vorticity(dd, cuda):
    """Known answer: a single 2D inviscid shearing vortex wave keeps its
    vorticity i(kx u_y - k_y(t) u_x) while u_y grows 8.5x as |k|^2 goes from 17
    to 2, with the pressure solve on the current k^2 (laplace_k2 = 'current')."""
    shape = (32, 32)
    S, kx, ky, A = 1.0, 1, 4, 1e-3
    G = dd.mods.IncompressibleHydro(shape, dd.mods.FourierShearRepresentation)
    G.parameters['shear_rate'] = S
    G.laplace_k2 = 'current'
    d = G.create_fields(0.)
    c = d['u'][0]
    y, x = c.xspace_grid()
    s = np.sin(kx * x + ky * y)
    d['u']['x']['xspace'] = -A * ky * s
    d['u']['y']['xspace'] = A * kx * s

    def vort():
        ux, uy = d['u']['x'].to_numpy('kspace'), d['u']['y'].to_numpy('kspace')
        kyt = d['u']['x'].k_host['y'][kx, ky]
        return 1j * (kx * uy[kx, ky] - kyt * ux[kx, ky]), uy[kx, ky]

    w0, u0 = vort()
    ti = dd.mods.RK4(G)
    for _ in range(300):
        ti.do_advance(d, 1e-2)
    w1, u1 = vort()
    assert abs(u1) > 3 * abs(u0)
    assert abs(w1 - w0) < 1e-8 * abs(w0), (w0, w1)


@pytest.mark.gpu
def test_shear_needs_a_shearing_representation(dd, cuda):
    G = dd.mods.IncompressibleHydro((16, 16), dd.mods.FourierRepresentation)
    G.parameters['shear_rate'] = 1.0
    d, k = G.create_fields(0.), G.create_fields(0.)
    with pytest.raises(ValueError):
        G.RHS(d, k)
