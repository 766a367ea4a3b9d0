"""Tile schedules of the fused 2D y passes (dd_plan_set_schedule), the knob
the ensemble autotuner turns: every variant keeps the default tile's radix
sequence, so an ensemble step is bitwise the same under each, and bad
arguments are rejected through the C ABI."""
import ctypes

import numpy as np
import pytest


@pytest.mark.gpu
@pytest.mark.parametrize("n", [64, 128, 256, 512])
def test_y_tile_variants_are_bitwise_equal(dd, cuda, n):
    sizes = [n, n, n]
    results = []
    for v in range(3):
        ens = dd.ensemble.BoussinesqEnsemble2D(sizes, nu=2e-3, kappa=2e-3)
        c = ens.classes[0]
        assert c.ysched_count() == 3
        c.set_ysched(v)
        ens.load_initial_conditions(seed=5)
        for r in range(len(sizes)):
            u = dd.init_cond.turbulence_2d((n, n), seed=40 + r, energy_target=1e-3)
            st = ens.run_state(r)
            ens.set_run_state(r, [u[0], u[1], st[2]])
        for _ in range(2):
            ens.step(1e-2, graph=(v != 1))
        results.append([np.stack(ens.run_state(r)) for r in range(len(sizes))])
    for v in (1, 2):
        for a, b in zip(results[v], results[0]):
            np.testing.assert_array_equal(a, b)


@pytest.mark.gpu
def test_schedule_abi_rejects_bad_arguments(dd, cuda):
    plan = dd.engine.Plan((64, 64), (2 * np.pi,) * 2)
    v, n = ctypes.c_int(-1), ctypes.c_int(-1)
    dd._lib.call("dd_plan_get_schedule", plan.handle, 0, ctypes.byref(v), ctypes.byref(n))
    assert (v.value, n.value) == (0, 3)
    with pytest.raises(ValueError):
        dd._lib.call("dd_plan_set_schedule", plan.handle, 0, 3)
    with pytest.raises(ValueError):
        dd._lib.call("dd_plan_set_schedule", plan.handle, 1, 0)
    plan3 = dd.engine.Plan((16, 16, 16), (2 * np.pi,) * 3)
    dd._lib.call("dd_plan_get_schedule", plan3.handle, 0, ctypes.byref(v), ctypes.byref(n))
    assert n.value == 1
