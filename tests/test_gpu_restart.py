"""Snapshots written by ``advance`` (every save_cadence iterations, as
time_step.py:101-151) and ``restart`` (utils/restart.py:33-99): the files
follow the reference's layout, and a restarted run continues bit for bit."""
import json
import os

import numpy as np
import pytest


@pytest.mark.gpu
def test_snapshot_cadence_and_restart_3d(dd, cuda, tmp_path, monkeypatch):
    import torch
    monkeypatch.chdir(tmp_path)
    M = dd.mods
    shape, dt = (16, 16, 16), 2e-3
    RHS = M.IncompressibleHydro(shape, M.FourierRepresentation)
    RHS.parameters['nu'] = 5e-3
    data = RHS.create_fields(0.)
    for i, c in enumerate(dd.init_cond.turbulence_3d(shape, seed=41)):
        data['u'][i]['kspace'] = c
    ti = M.RK4(RHS)
    ti.save_cadence = 2
    for _ in range(5):
        ti.advance(data, dt)
    assert sorted(os.listdir(".")) == ["snap_00000", "snap_00001", "snap_00002"]
    snap = tmp_path / "snap_00002"
    assert sorted(os.listdir(snap)) == ["data.cpu0000.npz", "dedalus_obj_0000.json", "forcing_functions.py"]
    z = np.load(snap / "data.cpu0000.npz")
    assert {"time", "fields/u/0", "fields/u/1", "fields/u/2", "fields/u/0@space"} <= set(z.files)
    assert abs(float(z["time"]) - 4 * dt) < 1e-15
    obj = json.load(open(snap / "dedalus_obj_0000.json"))
    assert obj["physics"]["class"] == "IncompressibleHydro" and obj["integrator"]["iteration"] == 4

    RHS2, data2, ti2 = M.restart(str(snap))
    assert ti2.iteration == 4 and abs(ti2.time - 4 * dt) < 1e-15 and ti2.save_cadence == 2
    assert RHS2.parameters['nu'] == 5e-3
    ti2.do_advance(data2, dt)
    for i in range(3):
        assert torch.equal(data2['u'][i].kdata, data['u'][i].kdata)


@pytest.mark.gpu
def test_restart_2d_boussinesq_with_xspace_component(dd, cuda, tmp_path, monkeypatch):
    import torch
    monkeypatch.chdir(tmp_path)
    M = dd.mods
    shape, dt = (64, 64), 1e-2
    RHS = M.BoussinesqHydro(shape, M.FourierRepresentation, length=(2 * np.pi, 4.0))
    RHS.parameters.update({'nu': 2e-3, 'kappa': 2e-3, 'boussinesq_direction': 'y', 'beta': 0.5})
    data = RHS.create_fields(0.)
    data['T'][0]['kspace'] = dd.init_cond.band_limited_noise_2d(shape, length=(2 * np.pi, 4.0), seed=42)
    ti = M.RK2mid(RHS)
    ti.save_cadence = 10
    for _ in range(3):
        ti.advance(data, dt)
    x = data['T'][0]['xspace'].clone()         # leave T in x-space for the snapshot
    ti.snapshot(data)
    RHS2, data2, ti2 = M.restart("snap_00001")
    assert RHS2.parameters['boussinesq_direction'] == 'y' and RHS2.parameters['beta'] == 0.5
    assert tuple(RHS2.length) == (2 * np.pi, 4.0)
    assert data2['T'][0]._curr_space == 'xspace'
    assert torch.equal(data2['T'][0].data, x)
    for _ in range(2):
        ti.do_advance(data, dt)
        ti2.do_advance(data2, dt)
    for f, c in [('u', 0), ('u', 1), ('T', 0)]:
        a = data[f][c].to_numpy('kspace')
        b = data2[f][c].to_numpy('kspace')
        assert np.array_equal(a, b), (f, c)
