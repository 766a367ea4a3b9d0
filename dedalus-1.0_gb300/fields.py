"""Field containers: the reference's TensorField / VectorField / ScalarField
classes bound to a representation (dedalus/data_objects/fields.py:35-245)
and ``StateData`` (dedalus/data_objects/state_data.py:45-145).  Component
order is x, y, z (fields.py:148-151).  HDF5 snapshot methods are out of
scope (see ``save_npz`` for a host dump of the state)."""
from collections import OrderedDict

import numpy as np
import torch


def create_field_classes(representation, shape, length):
    """fields.py:35-57: bind representation, shape and length to field types."""
    attr_dict = {'representation': representation, 'shape': shape, 'length': length}
    return {'TensorField': type('TensorField', (TensorFieldBase,), dict(attr_dict)),
            'VectorField': type('VectorField', (VectorFieldBase,), dict(attr_dict)),
            'ScalarField': type('ScalarField', (ScalarFieldBase,), dict(attr_dict))}


class BaseField:
    def __init__(self, sd, ncomp):
        self.sd = sd
        self.ncomp = ncomp
        self.ndim = len(self.shape)
        self.components = [self.representation(self.sd, self.shape, self.length) for _ in range(self.ncomp)]
        self.ctrans = {}

    def __getitem__(self, item):
        if type(item) == str:
            item = self.ctrans[item]
        return self.components[item]

    def __setitem__(self, item, data):
        if type(item) == str:
            item = self.ctrans[item]
        self.components[item] = data

    def __iter__(self):
        for i in range(self.ncomp):
            yield (i, self.components[i])

    def zero(self, comp, space='kspace'):
        if type(comp) == str:
            comp = self.ctrans[comp]
        self.components[comp][space] = 0.

    def zero_all(self, space='kspace'):
        for c in self.components:
            c[space] = 0.

    def report_counts(self):
        return [(c.fwd_count, c.rev_count) for c in self.components]


class TensorFieldBase(BaseField):
    def __init__(self, sd):
        BaseField.__init__(self, sd, sd.ndim ** 2)


class VectorFieldBase(BaseField):
    def __init__(self, sd):
        BaseField.__init__(self, sd, sd.ndim)
        if self.ncomp == 2:
            self.ctrans = {'x': 0, 0: 'x', 'y': 1, 1: 'y'}
        else:
            self.ctrans = {'x': 0, 0: 'x', 'y': 1, 1: 'y', 'z': 2, 2: 'z'}

    def max_square(self):
        """fields.py:153-157 (single device: no reduction across ranks).  As
        in the reference, reading c['xspace'] leaves every component in grid
        space; the maximum is one device reduction (dd_max_square)."""
        from . import _lib
        from .engine import current_stream, dptr
        comps = [c for i, c in self]
        for c in comps:
            c.require_space('xspace')
        out = torch.empty((), dtype=torch.float64, device=comps[0].device)
        xp, _keep = _lib.ptr_array([c.xdata.data_ptr() for c in comps])
        _lib.call("dd_max_square", len(comps), xp, comps[0].xdata.numel(), dptr(out), current_stream())
        return float(out.item())

    def div_free(self):
        """Project off the irrotational part (fields.py:169-195)."""
        comps = [c for i, c in self]
        for c in comps:
            c.require_space('kspace')
        k = comps[0].k_host
        names = [self.ctrans[i] for i in range(self.ncomp)]
        kk = [np.broadcast_to(k[n], comps[0].kdata.shape) for n in names]
        data = [c.kdata.cpu().numpy() for c in comps]
        divF = 0
        for i in range(self.ncomp):
            divF = divF + data[i] * (1j * k[names[i]])
        k2 = np.zeros(comps[0].kdata.shape)
        for v in k.values():
            k2 += v ** 2
        k2[k2 == 0] = 1.
        for i, c in enumerate(comps):
            data[i] -= -1j * k[names[i]] * divF / k2
            c['kspace'] = data[i]


class ScalarFieldBase(BaseField):
    def __init__(self, sd):
        BaseField.__init__(self, sd, 1)
        self.ctrans = {'': 0, 0: ''}

    def __getitem__(self, item):
        if item == 0:
            return self.components[0]
        return self.components[0][item]

    def __setitem__(self, item, data):
        if item == 0:
            self.components[0] = data
        else:
            self.components[0][item] = data

    def __getattr__(self, attr):
        if attr == 'components':
            raise AttributeError(attr)
        return getattr(self.components[0], attr)

    def zero(self, space='kspace'):
        self.components[0][space] = 0.


class StateData:
    """state_data.py:45-145."""

    def __init__(self, time, shape, length, field_class_dict, field_list=(), params=None):
        self.time = time
        self.shape = shape
        self.ndim = len(self.shape)
        self.length = length
        self._field_classes = field_class_dict
        self.parameters = {} if params is None else params
        self.fields = OrderedDict()
        for name, ftype in field_list:
            self.add_field(name, ftype)

    def __getitem__(self, item):
        return self.fields[item]

    def __iter__(self):
        for name, field in self.fields.items():
            yield (name, field)

    def clone(self):
        return self.__class__(self.time, self.shape, self.length, self._field_classes, params=self.parameters)

    def set_time(self, time):
        # state_data.py:117-121: shearing-box components follow the time
        self.time = time
        for name, field in self.fields.items():
            if not field.representation._static_k:
                for i, c in field:
                    c._update_k()

    def add_field(self, name, fieldtype):
        if name in self.fields:
            raise ValueError("Field with this name already exists.")
        self.fields[name] = self._field_classes[fieldtype](self)

    def save_npz(self, path):
        """Host dump of every component in its current space (the checkpoint
        analogue of StateData.snapshot, state_data.py:147-160)."""
        out = {'time': np.float64(self.time)}
        for name, field in self:
            for i, c in field:
                out['%s/%d/%s' % (name, i, c._curr_space)] = c.data.detach().cpu().numpy()
        np.savez(path, **out)

    def load_npz(self, path):
        z = np.load(path)
        self.time = float(z['time'])
        for key in z.files:
            if key == 'time':
                continue
            name, i, space = key.split('/')
            self.fields[name][int(i)][space] = z[key]
