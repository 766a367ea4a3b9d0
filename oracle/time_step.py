"""CPU oracle -- test infrastructure only.

Restatement of the reference's time integrators
(``dedalus/time_stepping/time_step.py``):

* ``TimeStepBase`` 48-179 (stop control, CFL dt); snapshots are I/O and are
  omitted (``snapshot`` is a no-op here).
* ``RK2mid`` 224-309 and ``RK2trap`` 312-392, as written, calling the C
  restatement of the reference's Cython stage kernels.
* ``RK4`` 395-483.  The reference's RK4 cannot run: ``RKBase.forward_step``
  (186-221) calls ``linear_step`` / ``intfac_step``, which are defined nowhere,
  and ``RHS(temp_data, temp_data)`` (449, 460, 471) would zero its own input
  (physics.py:140-142).  This restatement fixes the definition used
  throughout the project: ``linear_step == euler`` and
  ``intfac_step == etd1`` with ``intfactor = -IF``; each stage's RHS goes to
  its own derivative buffer; stages are
      k1 = N(y); y2 = etd1(y, k1, dt/2); k2 = N(y2); y3 = etd1(y, k2, dt/2);
      k3 = N(y3); y4 = etd1(y, k3, dt); k4 = N(y4);
      y+ = etd1(y, k1/6 + k2/3 + k3/3 + k4/6, dt)
  with the increments accumulated in the reference's order (434-474).
"""
import time

import numpy as np

from ._cstage import stage2d, stage3d


class TimeStepBase:
    """time_step.py:48-179."""

    def __init__(self, RHS, CFL=0.1, int_factor=None):
        self.RHS = RHS
        self.CFL = CFL
        self.int_factor = int_factor
        self.sim_stop_time = 1000
        self.wall_stop_time = 60. * 60.
        self.stop_iteration = 1000
        self.save_cadence = 100
        self.max_save_period = 100.
        self.time = 0
        self.iteration = 0
        self._nsnap = 0
        self._tlastsnap = 0.
        self.dt_old = np.finfo('d').max / 10.
        self._start_time = time.time()

    @property
    def ok(self):
        if self.iteration >= self.stop_iteration:
            return False
        if self.time >= self.sim_stop_time:
            return False
        if (time.time() - self._start_time) >= self.wall_stop_time:
            return False
        return True

    def advance(self, data, dt=None):
        if dt is None:
            dt = self.cfl_dt(data)
        self.do_advance(data, dt)

    def do_advance(self, data, dt):
        raise NotImplementedError("do_advance must be provided by subclass.")

    def snapshot(self, data):
        pass

    def cfl_dt(self, data):
        dt = self.CFL * self.RHS.compute_dt(data)
        if dt > 1.05 * self.dt_old:
            dt = 1.05 * self.dt_old
        self.dt_old = dt
        return dt

    def _kernels(self):
        return stage2d if self.RHS.ndim == 2 else stage3d


class RKBase(TimeStepBase):
    def linear_step(self, start, deriv, output, dt):
        self._kernels().euler(start, output, deriv, dt)

    def intfac_step(self, start, deriv, output, intfactor, dt):
        self._kernels().etd1(start, output, deriv, -intfactor, dt)

    def forward_step(self, start, deriv, output, dt):
        # time_step.py:187-221
        for fname, field in output:
            for cindex, comp in field:
                if deriv[fname][cindex].integrating_factor is None:
                    self.linear_step(start[fname][cindex]['kspace'],
                                     deriv[fname][cindex]['kspace'],
                                     comp['kspace'], dt)
                else:
                    self.intfac_step(start[fname][cindex]['kspace'],
                                     deriv[fname][cindex]['kspace'],
                                     comp['kspace'],
                                     deriv[fname][cindex].integrating_factor, dt)
        output.set_time(start.time + dt)


class RK2mid(RKBase):
    """time_step.py:224-309."""

    def __init__(self, *arg, **kwargs):
        TimeStepBase.__init__(self, *arg, **kwargs)
        self.data2 = self.RHS.create_fields(0.)
        self.deriv1 = self.RHS.create_fields(0.)
        self.deriv2 = self.RHS.create_fields(0.)
        k = self._kernels()
        self.euler, self.etd1, self.etd2rk2 = k.euler, k.etd1, k.etd2rk2

    def do_advance(self, data, dt):
        s = 'kspace'
        data2, deriv1, deriv2 = self.data2, self.deriv1, self.deriv2
        self.RHS.RHS(data, deriv1)
        for f in data.fields.keys():
            for c in range(data[f].ncomp):
                IF = deriv1[f][c].integrating_factor
                if IF is None:
                    self.euler(data[f][c][s], data2[f][c][s], deriv1[f][c][s], dt / 2.)
                else:
                    self.etd1(data[f][c][s], data2[f][c][s], deriv1[f][c][s], -IF, dt / 2.)
        data2.set_time(data.time + dt / 2.)
        self.RHS.RHS(data2, deriv2)
        for f in data.fields.keys():
            for c in range(data[f].ncomp):
                IF = deriv1[f][c].integrating_factor
                if IF is None:
                    self.euler(data[f][c][s], data[f][c][s], deriv2[f][c][s], dt)
                else:
                    self.etd2rk2(data[f][c][s], data[f][c][s], deriv1[f][c][s],
                                 deriv2[f][c][s], -IF, dt)
        data.set_time(data.time + dt)
        self.time += dt
        self.iteration += 1


class RK2trap(RKBase):
    """time_step.py:312-392."""

    def __init__(self, *arg, **kwargs):
        TimeStepBase.__init__(self, *arg, **kwargs)
        self.deriv1 = self.RHS.create_fields(0.)
        self.deriv2 = self.RHS.create_fields(0.)
        k = self._kernels()
        self.euler, self.etd1, self.etd2rk1 = k.euler, k.etd1, k.etd2rk1

    def do_advance(self, data, dt):
        s = 'kspace'
        deriv1, deriv2 = self.deriv1, self.deriv2
        self.RHS.RHS(data, deriv1)
        for f in data.fields.keys():
            for c in range(data[f].ncomp):
                IF = deriv1[f][c].integrating_factor
                if IF is None:
                    self.euler(data[f][c][s], data[f][c][s], deriv1[f][c][s], dt)
                else:
                    self.etd1(data[f][c][s], data[f][c][s], deriv1[f][c][s], -IF, dt)
        data.set_time(data.time + dt)
        self.RHS.RHS(data, deriv2)
        for f in data.fields.keys():
            for c in range(data[f].ncomp):
                IF = deriv1[f][c].integrating_factor
                if IF is None:
                    self.euler(data[f][c][s], data[f][c][s],
                               deriv2[f][c][s] - deriv1[f][c][s], dt / 2.)
                else:
                    self.etd2rk1(data[f][c][s], data[f][c][s], deriv1[f][c][s],
                                 deriv2[f][c][s], -IF, dt)
        self.time += dt
        self.iteration += 1


class RK4(RKBase):
    """time_step.py:395-483 with the stage definition in the module docstring."""

    def __init__(self, *arg, **kwargs):
        TimeStepBase.__init__(self, *arg, **kwargs)
        self.temp_data = self.RHS.create_fields(0.)
        self.temp_deriv = self.RHS.create_fields(0.)
        self.total_deriv = self.RHS.create_fields(0.)

    def do_advance(self, data, dt):
        temp, kd, total = self.temp_data, self.temp_deriv, self.total_deriv
        # k1
        self.RHS.RHS(data, kd)
        for fname, field in total:
            for cindex, comp in field:
                comp['kspace'] = kd[fname][cindex]['kspace'] / 6.
                comp.integrating_factor = kd[fname][cindex].integrating_factor
        # k2
        self.forward_step(data, kd, temp, dt / 2.)
        self.RHS.RHS(temp, kd)
        for fname, field in total:
            for cindex, comp in field:
                comp['kspace'] += kd[fname][cindex]['kspace'] / 3.
        # k3
        self.forward_step(data, kd, temp, dt / 2.)
        self.RHS.RHS(temp, kd)
        for fname, field in total:
            for cindex, comp in field:
                comp['kspace'] += kd[fname][cindex]['kspace'] / 3.
        # k4
        self.forward_step(data, kd, temp, dt)
        self.RHS.RHS(temp, kd)
        for fname, field in total:
            for cindex, comp in field:
                comp['kspace'] += kd[fname][cindex]['kspace'] / 6.
        # complete step
        self.forward_step(data, total, data, dt)
        self.time += dt
        self.iteration += 1
