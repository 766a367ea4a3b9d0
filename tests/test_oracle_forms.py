"""The divergence forms of the nonlinear terms (the CUDA path's physics 2 / 3
in 3D and 2 / 3 in 2D) restated in numpy and checked on the CPU against the
oracle's reference-order right-hand sides on solenoidal states:

* 3D hydro: P[-i k_j T_ij], T = u u^T - u_z^2 I (five products), equals
  P[-(u.grad)u];
* 3D MHD: P[-i k_j M_ij], M = u u^T - B B^T / (4 pi rho0) - M_zz I, equals
  P[-(u.grad)u + (J x B) / (4 pi rho0)]; the induction term is unchanged;
* 2D Boussinesq: P[-i k_j T_ij] (two products) plus buoyancy, and
  -i k . (u T) - beta u_y for the temperature, equal the reference terms;
* a state with a divergent part breaks the equality (which is why the CUDA
  path checks every state before it takes these forms).
Transforms and products are the oracle's own (numpy FFT, 2/3 rule)."""
import numpy as np
import pytest

from oracle import physics as OP
from oracle.representation import FourierRepresentation as R


def _rel(a, b):
    num = sum(np.sum(np.abs(x - y) ** 2) for x, y in zip(a, b))
    den = sum(np.sum(np.abs(y) ** 2) for y in b)
    return float(np.sqrt(num / den))


def _solenoidal(shape, seed, comps, k):
    rng = np.random.Generator(np.random.PCG64(seed))
    u = []
    for _ in range(comps):
        x = rng.normal(size=shape)
        kd = np.transpose(np.fft.rfftn(x / x.size), [1, 0, 2][:len(shape)])
        u.append(kd)
    names = ['x', 'y', 'z'][:comps]
    k2 = sum(np.broadcast_to(k[n], u[0].shape) ** 2 for n in names)
    d = sum(k[n] * u[i] for i, n in enumerate(names)) / np.where(k2 == 0, 1, k2)
    return [u[i] - k[n] * d for i, n in enumerate(names)]


def _project(N, k, names):
    k2 = sum(np.broadcast_to(k[n], N[0].shape) ** 2 for n in names)
    d = sum(k[n] * N[i] for i, n in enumerate(names)) / np.where(k2 == 0, 1, k2)
    return [N[i] - k[n] * d for i, n in enumerate(names)]


def _state(P, fields):
    data = P.create_fields(0.)
    for (f, c), a in fields.items():
        data[f][c]['kspace'] = a.copy()
    return data


def _to_x(comp, a):
    comp['kspace'] = a.copy()
    return comp['xspace'].copy()


def _to_k(comp, x):
    comp['xspace'] = x
    return comp['kspace'].copy()


def _div_k(k, names, T):
    """-i k_j T_ij for a symmetric tensor given as a dict {(i, j): k array}."""
    out = []
    for i, a in enumerate(names):
        s = 0
        for j, b in enumerate(names):
            t = T.get((i, j), T.get((j, i)))
            if t is not None:
                s = s + k[b] * t
        out.append(-1j * s)
    return out


@pytest.mark.parametrize("divergent", [False, True])
def test_3d_hydro_divergence_form(divergent):
    shape = (16, 16, 16)
    P = OP.IncompressibleHydro(shape, R)
    P.parameters['nu'] = 0.
    probe = P.create_fields(0.)['u'][0]
    k = probe.k
    u = _solenoidal(shape, 1, 3, k)
    if divergent:
        u[0] = u[0] + 0.2 * np.where(np.abs(np.broadcast_to(k['x'], u[0].shape)) > 0, 1j, 0) * u[1]
    data = _state(P, {('u', i): u[i] for i in range(3)})
    deriv = P.create_fields(0.)
    P.RHS(data, deriv)
    ref = [deriv['u'][i]['kspace'] for i in range(3)]
    ux = [_to_x(probe, a) for a in u]
    T = {(0, 0): ux[0] ** 2 - ux[2] ** 2, (1, 1): ux[1] ** 2 - ux[2] ** 2,
         (0, 1): ux[0] * ux[1], (0, 2): ux[0] * ux[2], (1, 2): ux[1] * ux[2]}
    Tk = {key: _to_k(probe, v) for key, v in T.items()}
    got = _project(_div_k(k, ['x', 'y', 'z'], Tk), k, ['x', 'y', 'z'])
    err = _rel(got, ref)
    assert (err > 1e-3) if divergent else (err < 1e-12), err


def test_3d_mhd_divergence_form():
    shape = (16, 16, 16)
    rho0 = 2.0
    fpr = 4 * np.pi * rho0
    P = OP.IncompressibleMHD(shape, R)
    P.parameters.update({'nu': 0., 'eta': 0., 'rho0': rho0})
    probe = P.create_fields(0.)['u'][0]
    k = probe.k
    u, B = _solenoidal(shape, 2, 3, k), _solenoidal(shape, 3, 3, k)
    data = _state(P, {**{('u', i): u[i] for i in range(3)}, **{('B', i): B[i] for i in range(3)}})
    deriv = P.create_fields(0.)
    P.RHS(data, deriv)
    ux = [_to_x(probe, a) for a in u]
    bx = [_to_x(probe, a) for a in B]
    m = {(i, j): ux[i] * ux[j] - bx[i] * bx[j] / fpr for i in range(3) for j in range(i, 3)}
    T = {(0, 0): m[(0, 0)] - m[(2, 2)], (1, 1): m[(1, 1)] - m[(2, 2)],
         (0, 1): m[(0, 1)], (0, 2): m[(0, 2)], (1, 2): m[(1, 2)]}
    Tk = {key: _to_k(probe, v) for key, v in T.items()}
    got = _project(_div_k(k, ['x', 'y', 'z'], Tk), k, ['x', 'y', 'z'])
    assert _rel(got, [deriv['u'][i]['kspace'] for i in range(3)]) < 1e-12
    # induction: curl(u x B) in both forms (the same products)
    uxb = [ux[1] * bx[2] - ux[2] * bx[1], ux[2] * bx[0] - ux[0] * bx[2], ux[0] * bx[1] - ux[1] * bx[0]]
    c = [_to_k(probe, v) for v in uxb]
    curl = [1j * (k['y'] * c[2] - k['z'] * c[1]), 1j * (k['z'] * c[0] - k['x'] * c[2]),
            1j * (k['x'] * c[1] - k['y'] * c[0])]
    assert _rel(curl, [deriv['B'][i]['kspace'] for i in range(3)]) < 1e-12


def test_2d_boussinesq_divergence_form():
    shape = (32, 32)
    P = OP.BoussinesqHydro(shape, R)
    P.parameters.update({'nu': 0., 'kappa': 0., 'g': 1.3, 'alpha_t': 0.7, 'beta': 0.9,
                         'boussinesq_direction': 'y'})
    probe = P.create_fields(0.)['u'][0]
    k = probe.k
    u = _solenoidal(shape, 4, 2, k)
    rng = np.random.Generator(np.random.PCG64(5))
    T = _to_k(probe, rng.normal(size=shape))
    data = _state(P, {('u', 0): u[0], ('u', 1): u[1], ('T', 0): T})
    deriv = P.create_fields(0.)
    P.RHS(data, deriv)
    ux = [_to_x(probe, a) for a in u]
    tx = _to_x(probe, T)
    Tk = {(0, 0): _to_k(probe, ux[0] ** 2 - ux[1] ** 2), (0, 1): _to_k(probe, ux[0] * ux[1])}
    N = _div_k(k, ['x', 'y'], Tk)
    N[1] = N[1] + T * 1.3 * 0.7
    got_u = _project(N, k, ['x', 'y'])
    flux = [_to_k(probe, ux[0] * tx), _to_k(probe, ux[1] * tx)]
    got_T = -(1j * (k['x'] * flux[0] + k['y'] * flux[1])) - u[1] * 0.9
    assert _rel(got_u + [got_T], [deriv['u'][0]['kspace'], deriv['u'][1]['kspace'], deriv['T']['kspace']]) < 1e-12
