"""GPU integrators: drop-ins for the reference's ``RK2mid``, ``RK2trap`` and
``RK4`` (dedalus/time_stepping/time_step.py:48-483).

Same constructor ``Cls(RHS, CFL=0.1, int_factor=None)``, ``advance(data,
dt=None)``, ``do_advance(data, dt)``, stop controls (``ok``,
``stop_iteration``, ``sim_stop_time``, ``wall_stop_time``), ``time``,
``iteration``, ``cfl_dt`` and ``final_stats``.

Two execution paths give the same result (to roundoff):
* fused: one C-ABI call per step (RK4 for 3D hydro: ``dd_hydro3d_rk4_step``),
  chosen automatically when the physics provides it;
* generic: ``RHS(data, deriv)`` plus the reference's stage kernels
  (``dd_euler``/``dd_etd1``/``dd_etd2rk1``/``dd_etd2rk2``) on the device,
  exactly as the reference sequences them.

RK4 follows the project's definition of the reference's unrunnable RK4
(``linear_step == euler``, ``intfac_step == etd1`` with ``-IF``, each stage's
RHS in its own buffer; see ``dd_hydro3d_rk4_step`` in include/dd_gb300.h).
"""
import ctypes
import time

import numpy as np
import torch

from . import _lib, restart
from .engine import current_stream, dptr


def _neg_if(comp):
    """Device copy of -integrating_factor (cached on the component)."""
    t = getattr(comp, '_neg_if_cache', None)
    IF = comp.integrating_factor
    if t is None or getattr(comp, '_neg_if_src', None) is not IF:
        host = IF.detach().cpu().numpy() if torch.is_tensor(IF) else np.asarray(IF)
        t = torch.from_numpy(np.ascontiguousarray(-host)).to(comp.device)
        comp._neg_if_cache = t
        comp._neg_if_src = IF
    return t


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
        self.wall_advance = 0.
        self.use_fused = True

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
        """time_step.py:101-107: snapshot when the iteration is a multiple of
        save_cadence or max_save_period has passed, then one step."""
        t0 = time.time()
        if (self.iteration % self.save_cadence) == 0 or (self.time - self._tlastsnap >= self.max_save_period):
            self.snapshot(data)
        if dt is None:
            dt = self.cfl_dt(data)
        self.do_advance(data, dt)
        self.wall_advance += time.time() - t0

    def do_advance(self, data, dt):
        raise NotImplementedError("do_advance must be provided by subclass.")

    def snapshot(self, data):
        """time_step.py:112-151: directory snap_%05i with the fields, the
        run description and the forcing sidecar (layout in restart.py)."""
        restart.save(restart.SNAP_DIR % self._nsnap, self.RHS, data, self)
        self._nsnap += 1
        self._tlastsnap = self.time

    def final_stats(self):
        if self.iteration:
            print("total advance wall time: %10.5e sec" % self.wall_advance)
            print("%10.5e sec/step " % (self.wall_advance / self.iteration))

    def finalize(self, data):
        self.final_stats()

    def cfl_dt(self, data):
        dt = self.CFL * self.RHS.compute_dt(data)
        if dt > 1.05 * self.dt_old:
            dt = 1.05 * self.dt_old
        self.dt_old = dt
        return dt

    # ------------------------------------------------------------ helpers
    @staticmethod
    def _k(comp):
        comp.require_space('kspace')
        return comp.kdata

    def _finish(self, dt):
        self.time += dt
        self.iteration += 1


class RKBase(TimeStepBase):
    def linear_step(self, start, deriv, output, dt):
        _lib.call("dd_euler", dptr(start), dptr(output), dptr(deriv), float(dt), start.numel(), current_stream())

    def intfac_step(self, start, deriv, output, neg_intfactor, dt):
        _lib.call("dd_etd1", start.dim(), dptr(start), dptr(output), dptr(deriv), dptr(neg_intfactor), float(dt),
                  start.numel(), current_stream())

    def forward_step(self, start, deriv, output, dt):
        # time_step.py:187-221
        for fname, field in output:
            for cindex, comp in field:
                d = deriv[fname][cindex]
                o = self._k(comp)
                if d.integrating_factor is None:
                    self.linear_step(self._k(start[fname][cindex]), self._k(d), o, dt)
                else:
                    self.intfac_step(self._k(start[fname][cindex]), self._k(d), o, _neg_if(d), dt)
        output.set_time(start.time + dt)


class RK2mid(RKBase):
    """time_step.py:224-309."""

    def __init__(self, *arg, **kwargs):
        TimeStepBase.__init__(self, *arg, **kwargs)
        self.data2 = self.RHS.create_fields(0.)
        self.deriv1 = self.RHS.create_fields(0.)
        self.deriv2 = self.RHS.create_fields(0.)

    def do_advance(self, data, dt):
        fused = getattr(self.RHS, 'fused_rk2mid', None) if self.use_fused else None
        if fused is not None and fused(data, dt, self):
            data.set_time(data.time + dt)
            return self._finish(dt)
        data2, deriv1, deriv2 = self.data2, self.deriv1, self.deriv2
        st = current_stream()
        self.RHS.RHS(data, deriv1)
        for f in data.fields.keys():
            for c in range(data[f].ncomp):
                d1 = deriv1[f][c]
                s, o, k1 = self._k(data[f][c]), self._k(data2[f][c]), self._k(d1)
                if d1.integrating_factor is None:
                    _lib.call("dd_euler", dptr(s), dptr(o), dptr(k1), dt / 2., s.numel(), st)
                else:
                    _lib.call("dd_etd1", s.dim(), dptr(s), dptr(o), dptr(k1), dptr(_neg_if(d1)), dt / 2.,
                              s.numel(), st)
        data2.set_time(data.time + dt / 2.)
        self.RHS.RHS(data2, deriv2)
        for f in data.fields.keys():
            for c in range(data[f].ncomp):
                d1 = deriv1[f][c]
                s, k1, k2 = self._k(data[f][c]), self._k(d1), self._k(deriv2[f][c])
                if d1.integrating_factor is None:
                    _lib.call("dd_euler", dptr(s), dptr(s), dptr(k2), float(dt), s.numel(), st)
                else:
                    _lib.call("dd_etd2rk2", s.dim(), dptr(s), dptr(s), dptr(k1), dptr(k2), dptr(_neg_if(d1)),
                              float(dt), s.numel(), st)
        data.set_time(data.time + dt)
        self._finish(dt)


class RK2trap(RKBase):
    """time_step.py:312-392."""

    def __init__(self, *arg, **kwargs):
        TimeStepBase.__init__(self, *arg, **kwargs)
        self.deriv1 = self.RHS.create_fields(0.)
        self.deriv2 = self.RHS.create_fields(0.)
        self._diff = None

    def do_advance(self, data, dt):
        deriv1, deriv2 = self.deriv1, self.deriv2
        st = current_stream()
        self.RHS.RHS(data, deriv1)
        for f in data.fields.keys():
            for c in range(data[f].ncomp):
                d1 = deriv1[f][c]
                s, k1 = self._k(data[f][c]), self._k(d1)
                if d1.integrating_factor is None:
                    _lib.call("dd_euler", dptr(s), dptr(s), dptr(k1), float(dt), s.numel(), st)
                else:
                    _lib.call("dd_etd1", s.dim(), dptr(s), dptr(s), dptr(k1), dptr(_neg_if(d1)), float(dt),
                              s.numel(), st)
        data.set_time(data.time + dt)
        self.RHS.RHS(data, deriv2)
        for f in data.fields.keys():
            for c in range(data[f].ncomp):
                d1 = deriv1[f][c]
                s, k1, k2 = self._k(data[f][c]), self._k(d1), self._k(deriv2[f][c])
                if d1.integrating_factor is None:
                    # euler(data, data, deriv2 - deriv1, dt/2)
                    if self._diff is None or self._diff.shape != s.shape:
                        self._diff = torch.empty_like(s)
                    _lib.call("dd_scale_add", dptr(k2), dptr(self._diff), 1.0, 0, s.numel(), st)
                    _lib.call("dd_scale_add", dptr(k1), dptr(self._diff), -1.0, 1, s.numel(), st)
                    _lib.call("dd_euler", dptr(s), dptr(s), dptr(self._diff), dt / 2., s.numel(), st)
                else:
                    _lib.call("dd_etd2rk1", s.dim(), dptr(s), dptr(s), dptr(k1), dptr(k2), dptr(_neg_if(d1)),
                              float(dt), s.numel(), st)
        self._finish(dt)


class RK4(RKBase):
    """time_step.py:395-483, with the stage definition in the module docstring."""

    def __init__(self, *arg, **kwargs):
        TimeStepBase.__init__(self, *arg, **kwargs)
        self._generic = None

    def _generic_buffers(self):
        if self._generic is None:
            self._generic = (self.RHS.create_fields(0.), self.RHS.create_fields(0.), self.RHS.create_fields(0.))
        return self._generic

    def do_advance(self, data, dt):
        fused = getattr(self.RHS, 'fused_rk4', None) if self.use_fused else None
        if fused is not None and fused(data, dt):
            data.set_time(data.time + dt)
            return self._finish(dt)
        temp, kd, total = self._generic_buffers()
        st = current_stream()

        def accumulate(w, first):
            for fname, field in total:
                for cindex, comp in field:
                    src = self._k(kd[fname][cindex])
                    _lib.call("dd_scale_add", dptr(src), dptr(self._k(comp)), float(w), 0 if first else 1,
                              src.numel(), st)
                    if first:
                        comp.integrating_factor = kd[fname][cindex].integrating_factor

        self.RHS.RHS(data, kd)
        accumulate(1. / 6., True)
        self.forward_step(data, kd, temp, dt / 2.)
        self.RHS.RHS(temp, kd)
        accumulate(1. / 3., False)
        self.forward_step(data, kd, temp, dt / 2.)
        self.RHS.RHS(temp, kd)
        accumulate(1. / 3., False)
        self.forward_step(data, kd, temp, dt)
        self.RHS.RHS(temp, kd)
        accumulate(1. / 6., False)
        self.forward_step(data, total, data, dt)
        self._finish(dt)
