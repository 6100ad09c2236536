"""Tiny unit system: angles, lengths, energies, time.

A ``Unit`` has a physical kind and a scale relative to the base unit of that
kind (rad, mm, keV, s).  ``number * unit`` gives a ``Quantity`` (an ndarray
subclass) whose ``.to(other).value`` rescales within the same kind.
"""
import math
from contextlib import contextmanager

import numpy as np


class UnitConversionError(Exception):
    pass


class Unit:
    # ndarray * unit -> Unit.__rmul__ (numpy defers), as astropy units do
    __array_ufunc__ = None

    def __init__(self, name, kind, scale):
        self.name = name
        self.kind = kind
        self.scale = scale

    def __rmul__(self, other):
        return Quantity(other, self)

    def __mul__(self, other):
        if isinstance(other, Unit):
            return Unit(self.name + '*' + other.name, (self.kind, '*', other.kind),
                        self.scale * other.scale)
        return Quantity(other, self)

    def __rtruediv__(self, other):
        return Quantity(other, Unit('1/' + self.name, ('1/', self.kind), 1. / self.scale))

    def __truediv__(self, other):
        if isinstance(other, Unit):
            return Unit(self.name + '/' + other.name, (self.kind, '/', other.kind),
                        self.scale / other.scale)
        return NotImplemented

    def __pow__(self, p):
        return Unit(self.name + '**%s' % p, (self.kind, '**', p), self.scale ** p)

    def to(self, other, value=1.0, equivalencies=None):
        return Quantity(value, self).to(other, equivalencies=equivalencies).value

    def __repr__(self):
        return 'Unit(%s)' % self.name

    def __eq__(self, other):
        return isinstance(other, Unit) and self.kind == other.kind and self.scale == other.scale

    def __hash__(self):
        return hash((str(self.kind), self.scale))


rad = Unit('rad', 'angle', 1.0)
deg = Unit('deg', 'angle', math.pi / 180.)
degree = deg
arcmin = Unit('arcmin', 'angle', math.pi / 180. / 60.)
arcsec = Unit('arcsec', 'angle', math.pi / 180. / 3600.)
mm = Unit('mm', 'length', 1.0)
um = Unit('um', 'length', 1e-3)
nm = Unit('nm', 'length', 1e-6)
cm = Unit('cm', 'length', 10.)
m = Unit('m', 'length', 1000.)
Angstrom = Unit('Angstrom', 'length', 1e-7)
keV = Unit('keV', 'energy', 1.0)
eV = Unit('eV', 'energy', 1e-3)
s = Unit('s', 'time', 1.0)
ks = Unit('ks', 'time', 1e3)
dimensionless_unscaled = Unit('', 'dimensionless', 1.0)

_HC_KEV_NM = 1.2398419843320026  # h*c in keV*nm


class Quantity(np.ndarray):
    def __new__(cls, value, unit=None, dtype=None, copy=True):
        if isinstance(value, Quantity) and unit is None:
            unit = value.unit
        arr = np.array(value, dtype=dtype if dtype is not None else float)
        obj = arr.view(cls)
        obj.unit = unit if unit is not None else dimensionless_unscaled
        return obj

    def __array_finalize__(self, obj):
        self.unit = getattr(obj, 'unit', dimensionless_unscaled)

    @property
    def value(self):
        v = self.view(np.ndarray)
        return v[()] if v.ndim == 0 else v

    def to(self, other, equivalencies=None):
        if self.unit.kind == other.kind:
            return Quantity(self.value * (self.unit.scale / other.scale), other)
        if equivalencies == 'spectral' or equivalencies is not None:
            kinds = {self.unit.kind, other.kind}
            if kinds == {'energy', 'length'}:
                # E [keV] * lambda [nm] = hc
                v = self.value * self.unit.scale
                out = _HC_KEV_NM / v
                return Quantity(out * (nm.scale / other.scale), other)
        raise UnitConversionError('%s -> %s' % (self.unit, other))

    def decompose(self):
        return self

    def __reduce__(self):
        return (Quantity, (self.value, self.unit))


def spectral():
    return 'spectral'


def dimensionless_angles():
    return 'dimensionless_angles'


@contextmanager
def set_enabled_equivalencies(eq):
    yield


def quantity_input(func=None, **kwargs):
    if func is not None and callable(func):
        return func

    def deco(f):
        return f
    return deco
