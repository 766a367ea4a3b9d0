"""CPU oracle -- test infrastructure only.

Restatement of the reference's field containers
(``dedalus/data_objects/fields.py:35-245``) and ``StateData``
(``dedalus/data_objects/state_data.py:45-145``).  Snapshot/HDF5 parts are
out of scope and omitted.
"""
from collections import OrderedDict

import numpy as np


def create_field_classes(representation, shape, length):
    """fields.py:35-57."""
    attr_dict = {'representation': representation, 'shape': shape, 'length': length}
    return {'TensorField': type('TensorField', (TensorFieldBase,), dict(attr_dict)),
            'VectorField': type('VectorField', (VectorFieldBase,), dict(attr_dict)),
            'ScalarField': type('ScalarField', (ScalarFieldBase,), dict(attr_dict))}


class BaseField:
    """fields.py:59-132."""

    def __init__(self, sd, ncomp):
        self.sd = sd
        self.ncomp = ncomp
        self.ndim = len(self.shape)
        self.components = [self.representation(self.sd, self.shape, self.length)
                           for _ in range(self.ncomp)]
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


class TensorFieldBase(BaseField):
    def __init__(self, sd):
        BaseField.__init__(self, sd, sd.ndim ** 2)


class VectorFieldBase(BaseField):
    """fields.py:141-195."""

    def __init__(self, sd):
        BaseField.__init__(self, sd, sd.ndim)
        if self.ncomp == 2:
            self.ctrans = {'x': 0, 0: 'x', 'y': 1, 1: 'y'}
        else:
            self.ctrans = {'x': 0, 0: 'x', 'y': 1, 1: 'y', 'z': 2, 2: 'z'}

    def max_square(self):
        return np.array([(c['xspace'] ** 2).max() for i, c in self]).max()

    def div_free(self):
        # fields.py:169-195
        divF = 0
        for i, c in self:
            divF = divF + c.deriv(self.ctrans[i])
        k2 = self[i].k2(no_zero=True)
        for i, c in self:
            c['kspace'] -= -1j * c.k[self.ctrans[i]] * divF / k2


class ScalarFieldBase(BaseField):
    """fields.py:197-245."""

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

    def zero_all(self, space='kspace'):
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
        return self.__class__(self.time, self.shape, self.length, self._field_classes,
                              params=self.parameters)

    def set_time(self, time):
        # state_data.py:117-121
        self.time = time
        for name, field in self.fields.items():
            if field.representation.__name__ == 'FourierShearRepresentation':
                for i, c in field:
                    c._update_k()

    def add_field(self, name, fieldtype):
        if name in self.fields:
            raise ValueError("Field with this name already exists.")
        self.fields[name] = self._field_classes[fieldtype](self)
