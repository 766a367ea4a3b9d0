"""GPU physics classes: drop-ins for the reference's ``IncompressibleHydro``,
``BoussinesqHydro`` and ``IncompressibleMHD`` (dedalus/physics/physics.py).

Same constructor ``Cls(shape, representation, length=None)``, the same
``parameters`` dictionary and defaults, ``create_fields(t)``,
``RHS(data, deriv)`` (fills ``deriv[f][c]['kspace']`` and sets each
component's ``integrating_factor`` on the first call, physics.py:504-522),
``compute_dt`` and the forcing setters.  The right-hand sides are computed by
fused CUDA kernels (one C-ABI call per RHS); the shearing box, rotation, 3D
Boussinesq and 2D MHD run the reference's operator sequence on CUDA kernels
(generic.py).  The passive tracer and forcing functions raise
NotImplementedError instead of running anywhere else.
"""
import ctypes

import numpy as np
import torch

from . import _lib
from .config import decfg, precision_code
from .engine import current_stream, dptr
from .fields import create_field_classes, StateData
from .generic import ReferenceOrderRHS


def _ptrs(tensors):
    return _lib.ptr_array([t.data_ptr() for t in tensors])


class Physics:
    """physics.py:42-158 (base): fields, parameters, aux equations, dt."""

    def __init__(self, shape, representation, length=None):
        self.shape = shape
        self._representation = representation
        self.length = length if length else (2 * np.pi,) * len(self.shape)
        self.ndim = len(self.shape)
        self.dims = range(self.ndim)
        self._field_list = []
        self._aux_field_list = []
        self.parameters = {}
        self.aux_eqns = {}
        self.forcing_functions = {}
        self._forcing_function_names = {}
        self._field_classes = create_field_classes(self._representation, self.shape, self.length)
        self._is_finalized = False
        self._tracer = decfg.getboolean('physics', 'use_tracer')
        self.k2 = None
        self._ws = None
        self._tables = {}

    def __getitem__(self, item):
        value = self.parameters.get(item, None)
        if value is None:
            raise KeyError
        return value

    def create_fields(self, time, field_list=None):
        if field_list is None:
            field_list = self._field_list
        return StateData(time, self.shape, self.length, self._field_classes, field_list=field_list,
                         params=self.parameters)

    def _finalize(self):
        self._is_finalized = True

    def _precision(self):
        """Transform precision code of this physics (FFT.precision)."""
        return precision_code()

    def compute_dt(self, data):
        self.dtlist = []
        self.set_dtlist(data)
        return min(self.dtlist)

    # --------------------------------------------------------- device data
    def plan(self, data):
        return next(iter(data.fields.values()))[0].plan

    def workspace(self, nbytes):
        if self._ws is None or self._ws.numel() < nbytes:
            self._ws = None
            self._ws = torch.empty(int(nbytes), dtype=torch.uint8, device=torch.device('cuda', torch.cuda.current_device()))
        return self._ws

    def inv_k2_table(self, plan):
        """1/q for integer squared wavenumbers q (q = 0 -> 1), or None."""
        if not plan.integer_k:
            return None
        key = ('inv_k2', id(plan))
        t = self._tables.get(key)
        if t is None:
            qmax = int(sum((n // 2) ** 2 for n in plan.xshape))
            q = np.arange(qmax + 1, dtype=np.float64)
            q[0] = 1.
            t = torch.from_numpy(1.0 / q).to(plan.device)
            self._tables[key] = t
        return t

    def phi_table(self, plan, nu, vo, h):
        """dd_phi_table for (nu, vo, h) on this grid (3D or 2D variant)."""
        key = ('phi', id(plan), float(nu), int(vo), float(h))
        t = self._tables.get(key)
        if t is None:
            qmax = int(sum((n // 2) ** 2 for n in plan.xshape))
            t = torch.empty((qmax + 1, 4), dtype=torch.float64, device=plan.device)
            _lib.call("dd_phi_table", plan.ndim, float(nu), int(vo), float(h), qmax, dptr(t), current_stream())
            if len(self._tables) > 64:
                self._tables = {k: v for k, v in self._tables.items() if k[0] == 'inv_k2'}
            self._tables[key] = t
        return t


class IncompressibleHydro(ReferenceOrderRHS, Physics):
    """physics.py:419-610."""

    def __init__(self, *args, **kwargs):
        Physics.__init__(self, *args, **kwargs)
        self._field_list.append(('u', 'VectorField'))
        self._aux_field_list.append(('mathscalar', 'ScalarField'))
        self._aux_field_list.append(('mathvector', 'VectorField'))
        self.parameters['viscosity_order'] = 1
        self.parameters['nu'] = 0.
        self.parameters['shear_rate'] = 0.
        self.parameters['Omega'] = None
        if self._tracer:
            self._field_list.append(('c', 'ScalarField'))
            self.parameters['c_diff'] = 0.
        self._trans = {0: 'x', 1: 'y', 2: 'z'}
        self._first_rhs = True

    def _finalize(self):
        # physics.py:484-502
        Physics._finalize(self)
        if self._tracer:
            raise NotImplementedError("the passive tracer is not in the CUDA path")
        if self.forcing_functions:
            raise NotImplementedError("forcing functions are not in the CUDA path")
        if self.parameters['shear_rate'] == 0.:
            self._shear = False
        else:
            self._shear = True
            if self._representation._static_k:
                raise ValueError("A shearing representation must be used if shear_rate is nonzero.")
        self._rotation = self.parameters['Omega'] is not None

    def _generic(self):
        """True when this RHS runs the reference-ordered operator sequence
        (generic.py) instead of a fused kernel: shear, rotation, a shearing
        representation, 3D Boussinesq, 2D MHD."""
        if not self._is_finalized:
            self._finalize()
        return self._shear or self._rotation or not self._representation._static_k or self._generic_only()

    def _generic_only(self):
        return False

    def _diffusivities(self):
        """(field name, coefficient) pairs whose IF is coeff * k2**vo."""
        return [('u', self.parameters['nu'])]

    def _setup_integrating_factors(self, deriv):
        # physics.py:504-522 (and the Boussinesq/MHD extensions)
        vo = self.parameters['viscosity_order']
        for fname, coeff in self._diffusivities():
            for cindex, comp in deriv[fname]:
                comp.integrating_factor = None if coeff == 0. else coeff * comp.k2() ** vo
                comp._if_coeff = float(coeff)

    def set_velocity_forcing(self, func):
        self.forcing_functions['VelocityForcing'] = func

    def _begin_rhs(self, data, deriv):
        if not self._is_finalized:
            self._finalize()
        # The reference sets the factors on the first deriv it is given only
        # (physics.py:538-540); a deriv that never received them gets them here
        # instead of failing later in the integrator.
        if self._first_rhs or not hasattr(next(iter(deriv.fields.values()))[0], 'integrating_factor'):
            self._setup_integrating_factors(deriv)
            self._first_rhs = False
        for fname, field in data:
            for i, c in field:
                c.require_space('kspace')
        deriv.set_time(data.time)

    def _mark_kspace(self, deriv):
        for fname, field in deriv:
            for i, c in field:
                c.data = c.kdata
                c._curr_space = 'kspace'

    # ------------------------------------------------------------ 3D
    _phys3d = 0

    def _state3d(self):
        return [('u', 0), ('u', 1), ('u', 2)]

    def _params3d(self):
        return None

    def _groups3d(self):
        return ['u']

    def RHS(self, data, deriv):
        """RHS(u) = P[-(u.grad)u] (physics.py:527-599), fused on the GPU (the
        shear / rotation branches in the reference's operator order)."""
        if self._generic():
            return self._generic_hydro(data, deriv, project=True)
        self._begin_rhs(data, deriv)
        plan = self.plan(data)
        if self.ndim != 3:
            return self._rhs2d(data, deriv, plan)
        self._rhs3d(data, deriv, plan)

    def _rhs3d(self, data, deriv, plan):
        prec = self._precision()
        n = ctypes.c_size_t()
        _lib.call("dd_rhs3d_workspace_size", plan.handle, self._phys3d, prec, ctypes.byref(n))
        ws = self.workspace(n.value)
        names = self._state3d()
        sp, _a = _ptrs([data[f][c].kdata for f, c in names])
        dp, _b = _ptrs([deriv[f][c].kdata for f, c in names])
        pp = self._params3d()
        ppa = None if pp is None else (ctypes.c_double * len(pp))(*pp)
        ik2 = self.inv_k2_table(plan)
        _lib.call("dd_rhs3d", plan.handle, self._phys3d, ppa, sp, dp, None if ik2 is None else dptr(ik2), prec, 1,
                  dptr(ws), ws.numel(), current_stream())
        self._mark_kspace(deriv)

    _fused3d = True

    def _rk4_args(self, data, dt):
        """Plan, precision, viscosity order, coefficients, 1/k^2 table and the
        phi-table pointer arrays of a fused 3D RK4 step."""
        names = self._state3d()
        for f, c in names:
            data[f][c].require_space('kspace')
        plan = self.plan(data)
        vo = int(self.parameters['viscosity_order'])
        coeffs = [float(self._coeff_of(g)) for g in self._groups3d()]
        ik2 = self.inv_k2_table(plan)
        th = tf = None
        keep = []
        if ik2 is not None:
            tabs_h = [self.phi_table(plan, cf, vo, dt / 2.) for cf in coeffs]
            tabs_f = [self.phi_table(plan, cf, vo, dt) for cf in coeffs]
            th, _h = _ptrs(tabs_h)
            tf, _f = _ptrs(tabs_f)
            keep = [tabs_h, tabs_f, _h, _f]
        sp, _a = _ptrs([data[f][c].kdata for f, c in names])
        keep.append(_a)
        cf = (ctypes.c_double * len(coeffs))(*coeffs)
        return plan, self._precision(), vo, cf, ik2, th, tf, sp, keep

    # 'auto': the fused 3D step uses the divergence form of the nonlinear
    # terms (dd_rk4_step3d physics 2 for hydro: 3 + 5 transforms per RHS
    # instead of 6 + 3; physics 3 for MHD: 6 + 8 instead of 12 + 6) whenever
    # every vector field of the state is solenoidal to |k.u| <= 1e-12 |k||u|
    # (1e-6 with FP32 transforms; dd_divergence_sums, re-checked whenever the
    # state changed outside the fused steps), and the curl forms otherwise;
    # both equal the reference's terms to roundoff on such states.
    # 'rotational' always uses the rotational form, and so does a step
    # captured into a CUDA graph (the check reads back to the host).
    nonlinear_form = 'auto'
    DIV_TOL2 = 1e-24
    # With FP32 transforms the step keeps its increments (and so the state's
    # divergence) at FP32 accuracy: a relative divergence up to 1e-6, below the
    # FP32 path's own error, still takes the divergence form.
    DIV_TOL2_FP32 = 1e-12

    def _step_phys3d(self, plan, prec, sp):
        """Physics code of dd_rk4_step3d for this step: the divergence form
        (hydro 0 -> 2, MHD 1 -> 3) when every vector field of the state is
        solenoidal to the tolerance."""
        if (self._phys3d not in (0, 1) or self.nonlinear_form != 'auto' or prec == _lib.DD_DF64
                or torch.cuda.is_current_stream_capturing()):
            return self._phys3d
        ngroups = len(self._groups3d())
        buf = self._tables.get('div_sums')
        if buf is None or buf.numel() < 2 * ngroups:
            buf = self._tables['div_sums'] = torch.empty(2 * ngroups, dtype=torch.float64, device=plan.device)
        base = ctypes.cast(sp, ctypes.c_void_p).value      # the pointer array (kept alive by the caller)
        for g in range(ngroups):
            gp = ctypes.cast(ctypes.c_void_p(base + 3 * g * ctypes.sizeof(ctypes.c_void_p)),
                             ctypes.POINTER(ctypes.c_void_p))
            _lib.call("dd_divergence_sums", plan.handle, gp, ctypes.c_void_p(buf.data_ptr() + 16 * g),
                      current_stream())
        v = buf.tolist()
        tol = self.DIV_TOL2_FP32 if prec == _lib.DD_FP32 else self.DIV_TOL2
        ok = all(v[2 * g] <= tol * v[2 * g + 1] for g in range(ngroups))
        return self._phys3d + 2 if ok else self._phys3d

    def _state_form3d(self, data, plan, prec, sp):
        """(physics code, non-kept flag) of a fused 3D step: the divergence
        form when the state is solenoidal (_step_phys3d), and whether any state
        component holds energy outside the kept modes (dd_any_nonkept; then the
        step decays those modes, as the reference's etd1 does).  A fused step
        keeps a solenoidal, dealiased state so, so the result is reused until a
        state component is read or written through the public API (its
        version moves) or replaced; inside a stream capture nothing is read back
        (curl forms, decay on)."""
        if torch.cuda.is_current_stream_capturing():
            return self._step_phys3d(plan, prec, sp), None
        comps = [data[f][c] for f, c in self._state3d()]
        key = (tuple((id(c), c._version, c.kdata.data_ptr()) for c in comps), prec, self.nonlinear_form)
        cached = getattr(self, '_form_cache', None)
        if cached is not None and cached[0] == key:
            return cached[1]
        phys = self._step_phys3d(plan, prec, sp)
        flag = self._tables.get('nonkept')
        if flag is None:
            flag = self._tables['nonkept'] = torch.zeros(1, dtype=torch.int32, device=plan.device)
        flag.zero_()
        _lib.call("dd_any_nonkept", plan.handle, len(comps), sp, dptr(flag), current_stream())
        val = (phys, ctypes.c_int(int(flag.item())))
        self._form_cache = (key, val)
        return val

    def fused_rk4(self, data, dt):
        """One fused RK4 step on the device (dd_rk4_step3d) for 3D hydro / MHD;
        returns False when this physics/grid has no fused step."""
        if self.ndim != 3 or not self._fused3d:
            return False
        if self._generic():
            return False
        plan, prec, vo, cf, ik2, th, tf, sp, keep = self._rk4_args(data, dt)
        phys, nonkept = self._state_form3d(data, plan, prec, sp)
        self.last_phys3d = phys
        n = ctypes.c_size_t()
        _lib.call("dd_rhs3d_workspace_size", plan.handle, phys, prec, ctypes.byref(n))
        ws = self.workspace(n.value)
        pp = self._params3d()
        ppa = None if pp is None else (ctypes.c_double * len(pp))(*pp)
        _lib.call("dd_rk4_step3d", plan.handle, phys, ppa, sp, None if ik2 is None else dptr(ik2), th, tf,
                  cf, vo, float(dt), prec, None if nonkept is None else ctypes.byref(nonkept), dptr(ws), ws.numel(),
                  current_stream())
        return True

    # ------------------------------------------------------------ 2D
    _phys2d = 0

    def _state_names(self):
        return [('u', 0), ('u', 1)]

    def _params2d(self):
        return None

    def _rhs2d(self, data, deriv, plan):
        prec = self._precision()
        n = ctypes.c_size_t()
        _lib.call("dd_rhs2d_workspace_size", plan.handle, 1, prec, ctypes.byref(n))
        ws = self.workspace(n.value)
        names = self._state_names()
        sp, _a = _ptrs([data[f][c].kdata for f, c in names])
        dp, _b = _ptrs([deriv[f][c].kdata for f, c in names])
        pp = self._params2d()
        ppa = None if pp is None else (ctypes.c_double * 4)(*pp)
        ik2 = self.inv_k2_table(plan)
        _lib.call("dd_rhs2d", plan.handle, self._phys2d, ppa, 1, sp, 0, dp, 0,
                  None if ik2 is None else dptr(ik2), prec, 1, dptr(ws), ws.numel(), current_stream())
        self._mark_kspace(deriv)

    def _coeff_of(self, fname):
        return dict(self._diffusivities())[fname]

    def fused_rk2mid(self, data, dt, ti=None):
        """One fused RK2mid step on the device (dd_rk2mid_step2d) for 2D
        hydro / Boussinesq; returns False when there is no fused step."""
        if self.ndim != 2 or type(self) not in (IncompressibleHydro, BoussinesqHydro):
            return False
        if self._generic():
            return False
        names = self._state_names()
        for f, c in names:
            data[f][c].require_space('kspace')
        plan = self.plan(data)
        prec = self._precision()
        vo = int(self.parameters['viscosity_order'])
        coeffs = [float(self._coeff_of(f)) for f, c in names]
        n = ctypes.c_size_t()
        _lib.call("dd_rhs2d_workspace_size", plan.handle, 1, prec, ctypes.byref(n))
        ws = self.workspace(n.value)
        ik2 = self.inv_k2_table(plan)
        th = tf = None
        keep = []
        if ik2 is not None:
            tabs_h = [self.phi_table(plan, cf, vo, dt / 2.) for cf in coeffs]
            tabs_f = [self.phi_table(plan, cf, vo, dt) for cf in coeffs]
            keep = tabs_h + tabs_f
            th, _h = _ptrs(tabs_h)
            tf, _f = _ptrs(tabs_f)
            keep += [_h, _f]
        sp, _a = _ptrs([data[f][c].kdata for f, c in names])
        pp = self._params2d()
        ppa = None if pp is None else (ctypes.c_double * 4)(*pp)
        nus = (ctypes.c_double * 3)(*(coeffs + [0.] * (3 - len(coeffs))))
        phys = self._phys2d
        # below 256^2 points a step is launch/latency bound: the check's host
        # read would cost more than the transform it saves
        if (self.nonlinear_form == 'auto' and not torch.cuda.is_current_stream_capturing()
                and int(np.prod(plan.xshape)) >= 256 * 256):
            buf = self._tables.get('div_sums')
            if buf is None:
                buf = self._tables['div_sums'] = torch.empty(2, dtype=torch.float64, device=plan.device)
            _lib.call("dd_divergence_sums2d", plan.handle, 1, dptr(data['u'][0].kdata), dptr(data['u'][1].kdata), 0,
                      dptr(buf), current_stream())
            num, den = buf.tolist()
            if num <= (self.DIV_TOL2_FP32 if prec == _lib.DD_FP32 else self.DIV_TOL2) * den:
                phys += 2
        self.last_phys2d = phys
        _lib.call("dd_rk2mid_step2d", plan.handle, phys, ppa, 1, sp, 0,
                  None if ik2 is None else dptr(ik2), th, tf, nus, vo, float(dt), prec, None,
                  dptr(ws), ws.numel(), current_stream())
        return True

    def max_abs_vel(self, data):
        return np.sqrt(data['u'].max_square())

    def set_dtlist(self, data):
        dx = data['u']['x'].dx().min()
        self.dtlist.append(dx / self.max_abs_vel(data))


class BoussinesqHydro(IncompressibleHydro):
    """physics.py:612-721."""

    _fused3d = False

    def __init__(self, *args, **kwargs):
        IncompressibleHydro.__init__(self, *args, **kwargs)
        self._field_list.append(('T', 'ScalarField'))
        self.parameters['kappa'] = 0.
        self.parameters['g'] = 1.
        self.parameters['alpha_t'] = 1.
        self.parameters['beta'] = 1.
        self.parameters['boussinesq_direction'] = decfg.get('physics', 'boussinesq_direction')

    def _diffusivities(self):
        return [('u', self.parameters['nu']), ('T', self.parameters['kappa'])]

    def set_thermal_forcing(self, func):
        self.forcing_functions['ThermalForcing'] = func

    _phys2d = 1

    def _state_names(self):
        return [('u', 0), ('u', 1), ('T', 0)]

    def _direction_index(self):
        d = self.parameters['boussinesq_direction']
        ctrans = {'x': 0, 'y': 1} if self.ndim == 2 else {'x': 0, 'y': 1, 'z': 2}
        if d not in ctrans:
            raise KeyError(d)   # as data['u'][d] does for a 2D VectorField (fields.py:148-151)
        return ctrans[d]

    def _params2d(self):
        return [float(self.parameters['g']), float(self.parameters['alpha_t']), float(self.parameters['beta']),
                float(self._direction_index())]

    def _generic_only(self):
        return self.ndim == 3

    def RHS(self, data, deriv):
        """physics.py:664-712, fused on the GPU (2D; 3D and the shear /
        rotation branches in the reference's operator order)."""
        self._direction_index()
        if self._generic():
            return self._generic_boussinesq(data, deriv)
        self._begin_rhs(data, deriv)
        self._rhs2d(data, deriv, self.plan(data))

    def set_dtlist(self, data):
        IncompressibleHydro.set_dtlist(self, data)
        dx = data['u']['x'].dx().min()
        N = np.sqrt(np.abs(self.parameters['alpha_t'] * self.parameters['g'] * self.parameters['beta']))
        self.dtlist.append(dx / N)


class IncompressibleMHD(IncompressibleHydro):
    """physics.py:724-836."""

    def __init__(self, *args, **kwargs):
        IncompressibleHydro.__init__(self, *args, **kwargs)
        self._field_list.append(('B', 'VectorField'))
        self._aux_field_list.append(('mathvector2', 'VectorField'))
        self.parameters['rho0'] = 1.
        self.parameters['eta'] = 0.

    def _diffusivities(self):
        return [('u', self.parameters['nu']), ('B', self.parameters['eta'])]

    _phys3d = 1

    def _state3d(self):
        return [('u', 0), ('u', 1), ('u', 2), ('B', 0), ('B', 1), ('B', 2)]

    def _params3d(self):
        return [float(self.parameters['rho0'])]

    def _groups3d(self):
        return ['u', 'B']

    def _generic_only(self):
        return self.ndim == 2

    def RHS(self, data, deriv):
        """physics.py:770-819, fused on the GPU (3D; 2D and the shear /
        rotation branches in the reference's operator order)."""
        if self._generic():
            return self._generic_mhd(data, deriv)
        self._begin_rhs(data, deriv)
        self._rhs3d(data, deriv, self.plan(data))

    def max_alfven_speed(self, data):
        fpr = 4 * np.pi * self.parameters['rho0']
        return np.sqrt(data['B'].max_square() / fpr)

    def set_dtlist(self, data):
        IncompressibleHydro.set_dtlist(self, data)
        dx = data['u']['x'].dx().min()
        self.dtlist.append(dx / self.max_alfven_speed(data))


class LESHydro(IncompressibleHydro):
    """IncompressibleHydro on an LES grid with a learned subgrid closure: the
    RHS is P[-(u.grad)u - div tau], tau predicted pointwise by the closure
    network (closure.MLPClosure) from the resolved velocity gradients.  With
    closure=None it is the unclosed (no-model) LES.  No counterpart in the
    reference; the closed RHS and RK4 step are dd_les_rhs3d /
    dd_les_rk4_step3d."""

    _PREC = {'fp64': _lib.DD_FP64, 'fp32': _lib.DD_FP32}

    def __init__(self, *args, closure=None, precision=None, **kwargs):
        IncompressibleHydro.__init__(self, *args, **kwargs)
        if self.ndim != 3:
            raise ValueError("the LES closure is three-dimensional")
        if precision is not None and precision not in self._PREC:
            raise NotImplementedError("LES precision must be 'fp64' or 'fp32'")
        self.closure = closure
        self.precision = precision

    def _precision(self):
        if self.precision is None:
            return IncompressibleHydro._precision(self)
        return self._PREC[self.precision]

    def _finalize(self):
        IncompressibleHydro._finalize(self)
        if self._shear or self._rotation or not self._representation._static_k:
            raise NotImplementedError("the LES closure runs without shear or rotation")

    def _les_ws(self, plan, prec):
        n = ctypes.c_size_t()
        _lib.call("dd_les_workspace_size", plan.handle, prec, ctypes.byref(n))
        return self.workspace(n.value)

    def _rhs3d(self, data, deriv, plan):
        if self.closure is None:
            return IncompressibleHydro._rhs3d(self, data, deriv, plan)
        prec = self._precision()
        ws = self._les_ws(plan, prec)
        names = self._state3d()
        sp, _a = _ptrs([data[f][c].kdata for f, c in names])
        dp, _b = _ptrs([deriv[f][c].kdata for f, c in names])
        ik2 = self.inv_k2_table(plan)
        cl = self.closure.struct()
        _lib.call("dd_les_rhs3d", plan.handle, sp, dp, None if ik2 is None else dptr(ik2), prec, 1,
                  ctypes.byref(cl), dptr(ws), ws.numel(), current_stream())
        self._mark_kspace(deriv)

    def fused_rk4(self, data, dt):
        if self.closure is None:
            return IncompressibleHydro.fused_rk4(self, data, dt)
        if not self._is_finalized:
            self._finalize()
        plan, prec, vo, cf, ik2, th, tf, sp, keep = self._rk4_args(data, dt)
        ws = self._les_ws(plan, prec)
        cl = self.closure.struct()
        _lib.call("dd_les_rk4_step3d", plan.handle, sp, None if ik2 is None else dptr(ik2), th, tf, cf, vo,
                  float(dt), prec, None, ctypes.byref(cl), dptr(ws), ws.numel(), current_stream())
        return True
