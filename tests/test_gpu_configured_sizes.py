"""Oracle parity at the benchmark configurations' own sizes.

* 3D incompressible hydro 256^3, nu = 5e-3, RK4, dt = 2e-3 (the headline):
  five consecutive steps, each started from the oracle's state after the
  previous one (so every comparison is one step, as "checked per step against
  the reference CPU path" asks), and a 200-step free trajectory at 64^3 with
  the bound asserted after every step.
* 3D incompressible MHD 256^3, nu = eta = 5e-3, RK4, dt = 1e-3: one FP64 step
  against the oracle, and the FP32 transform path's per-field error against
  the same oracle step.
* 2D Boussinesq (direction y, N^2 = 1, nu = kappa = 2e-3) at 512^2, single
  run, and an uneven ensemble with all four configured sizes 64^2 .. 512^2,
  every run against its own oracle run.

Tolerances: FP64 <= 1e-12 relative L2 over all fields per step (free
trajectories: 1e-12 times the number of steps); FP32 transforms <= 1e-5 per
field (the FP32 bound used throughout the tests)."""
import numpy as np
import pytest

from oracle import physics as OP, time_step as OT
from oracle.representation import FourierRepresentation as OracleRep


def rel_l2(got, ref):
    num = sum(np.sum(np.abs(g - r) ** 2) for g, r in zip(got, ref))
    den = sum(np.sum(np.abs(r) ** 2) for r in ref)
    return float(np.sqrt(num / den))


def make_pair(dd, cls_name, shape, params, fields):
    M = dd.mods
    ro = getattr(OP, cls_name)(shape, OracleRep)
    rg = getattr(M, cls_name)(shape, M.FourierRepresentation)
    for r in (ro, rg):
        r.parameters.update(params)
    do, dg = ro.create_fields(0.), rg.create_fields(0.)
    for (f, c), a in fields:
        do[f][c]['kspace'] = a.copy()
        dg[f][c]['kspace'] = a
    return ro, do, rg, dg


def host(data, names, gpu):
    return [data[f][c].to_numpy('kspace') if gpu else data[f][c]['kspace'].copy() for f, c in names]


U3 = [('u', 0), ('u', 1), ('u', 2)]
MHD = U3 + [('B', 0), ('B', 1), ('B', 2)]
BOU = [('u', 0), ('u', 1), ('T', 0)]
BPAR = {'nu': 2e-3, 'kappa': 2e-3, 'g': 1., 'alpha_t': 1., 'beta': 1., 'boussinesq_direction': 'y'}


@pytest.mark.gpu
def test_hydro_256_five_steps_reseeded_from_oracle(dd, cuda):
    shape = (256, 256, 256)
    u0 = dd.init_cond.turbulence_3d(shape, seed=0)
    ro, do, rg, dg = make_pair(dd, 'IncompressibleHydro', shape, {'nu': 5e-3}, list(zip(U3, u0)))
    to, tg = OT.RK4(ro), dd.mods.RK4(rg)
    errs = []
    for step in range(5):
        if step:
            for (f, c), a in zip(U3, host(do, U3, False)):
                dg[f][c]['kspace'] = a                  # start from the oracle's state
        to.do_advance(do, 2e-3)
        tg.do_advance(dg, 2e-3)
        errs.append(rel_l2(host(dg, U3, True), host(do, U3, False)))
        assert rg.last_phys3d == 2                      # the benchmarked (divergence) form
    print("per-step rel L2 at 256^3:", errs)
    assert max(errs) < 1e-12, errs


@pytest.mark.gpu
def test_hydro_64_200_step_trajectory(dd, cuda):
    shape = (64, 64, 64)
    u0 = dd.init_cond.turbulence_3d(shape, seed=0)
    ro, do, rg, dg = make_pair(dd, 'IncompressibleHydro', shape, {'nu': 5e-3}, list(zip(U3, u0)))
    _r1, _d1, rs, ds = make_pair(dd, 'IncompressibleHydro', shape, {'nu': 5e-3}, list(zip(U3, u0)))
    to, tg, ts = OT.RK4(ro), dd.mods.RK4(rg), dd.mods.RK4(rs)
    worst_traj = worst_step = 0.0
    for step in range(200):
        prev = host(do, U3, False)
        to.do_advance(do, 2e-3)
        tg.do_advance(dg, 2e-3)
        for (f, c), a in zip(U3, prev):
            ds[f][c]['kspace'] = a                      # one step from the oracle's previous state
        ts.do_advance(ds, 2e-3)
        ref = host(do, U3, False)
        e_traj = rel_l2(host(dg, U3, True), ref)
        e_step = rel_l2(host(ds, U3, True), ref)
        assert e_step < 1e-12, (step, e_step)
        assert e_traj < 1e-12 * (step + 1), (step, e_traj)
        worst_traj, worst_step = max(worst_traj, e_traj), max(worst_step, e_step)
    assert tg.iteration == 200 and abs(dg.time - 0.4) < 1e-12
    print("64^3, 200 steps: worst one-step %.3e, trajectory %.3e" % (worst_step, worst_traj))


@pytest.mark.gpu
def test_mhd_256_fp64_step_and_fp32_per_field(dd, cuda):
    shape = (256, 256, 256)
    u = dd.init_cond.turbulence_3d(shape, seed=0, k0=3.0)
    b = dd.init_cond.turbulence_3d(shape, seed=1000, k0=3.0)
    params = {'nu': 5e-3, 'eta': 5e-3}
    ro, do, rg, dg = make_pair(dd, 'IncompressibleMHD', shape, params, list(zip(MHD, u + b)))
    OT.RK4(ro).do_advance(do, 1e-3)
    ref = host(do, MHD, False)
    del ro, do
    dd.mods.RK4(rg).do_advance(dg, 1e-3)
    assert rg.last_phys3d == 3                          # the benchmarked (divergence) form
    e64 = rel_l2(host(dg, MHD, True), ref)
    assert e64 < 1e-12, e64
    del rg, dg
    dd.config.decfg.set('FFT', 'precision', 'fp32')
    try:
        M = dd.mods
        r32 = M.IncompressibleMHD(shape, M.FourierRepresentation)
        r32.parameters.update(params)
        d32 = r32.create_fields(0.)
        for (f, c), a in zip(MHD, u + b):
            d32[f][c]['kspace'] = a
        M.RK4(r32).do_advance(d32, 1e-3)
    finally:
        dd.config.decfg.set('FFT', 'precision', 'fp64')
    got = host(d32, MHD, True)
    per_field = {"%s_%s" % (f, "xyz"[c]): rel_l2([g], [r]) for (f, c), g, r in zip(MHD, got, ref)}
    print("MHD 256^3 FP64 step rel L2 %.3e; FP32 per field %s" % (e64, per_field))
    for name, e in per_field.items():
        assert e < 1e-5, (name, e)


@pytest.mark.gpu
def test_boussinesq_512_single_run(dd, cuda):
    shape = (512, 512)
    T = dd.init_cond.band_limited_noise_2d(shape, seed=3)
    uu = dd.init_cond.turbulence_2d(shape, seed=4, energy_target=1e-2)
    ro, do, rg, dg = make_pair(dd, 'BoussinesqHydro', shape, BPAR, list(zip(BOU, [uu[0], uu[1], T])))
    to, tg = OT.RK2mid(ro), dd.mods.RK2mid(rg)
    for step in range(5):
        to.do_advance(do, 1e-2)
        tg.do_advance(dg, 1e-2)
        e = rel_l2(host(dg, BOU, True), host(do, BOU, False))
        assert e < 1e-12, (step, e)
    assert rg.last_phys2d == 3                          # divergence form (solenoidal u)


@pytest.mark.gpu
def test_ensemble_with_all_configured_sizes(dd, cuda):
    """Runs of 64^2, 128^2, 256^2 and 512^2 (two of the larger ones) in one
    graph-launched ensemble, configured as the benchmark's (u = 0, band-limited
    temperature noise, dt = 1e-2), each against its own oracle run."""
    sizes = [512, 64, 256, 128, 512, 256]
    dt, nsteps = 1e-2, 4
    ens = dd.ensemble.BoussinesqEnsemble2D(sizes, nu=2e-3, kappa=2e-3)
    ens.load_initial_conditions(seed=17)
    init = [ens.run_state(r) for r in range(len(sizes))]
    for _ in range(nsteps):
        ens.step(dt, graph=True)
    assert all(c.phys == 3 for c in ens.classes)
    for r, n in enumerate(sizes):
        rhs = OP.BoussinesqHydro((n, n), OracleRep)
        rhs.parameters.update(BPAR)
        d = rhs.create_fields(0.)
        for (f, c), a in zip(BOU, init[r]):
            d[f][c]['kspace'] = a.copy()
        ti = OT.RK2mid(rhs)
        for _ in range(nsteps):
            ti.do_advance(d, dt)
        e = rel_l2(ens.run_state(r), host(d, BOU, False))
        assert e < 1e-12, (r, n, e)
