"""Tiny unit system (test-only stand-in): angles, lengths, energies, time.

A ``Unit`` has a dimension (exponents of angle, length, energy and time) and
a scale relative to the base units rad, mm, keV and s.  ``number * unit``
gives a ``Quantity`` (an ndarray subclass) that carries its unit through
numpy arithmetic: products, quotients and powers combine units; sums,
differences, clipping and comparisons express the second operand in the
first one's unit; exp/log/arcsin/... take dimensionless values (the scale of
a ratio such as mm/um applied to the value first) and sin/cos/tan take
angles.  ``.to(other)`` rescales between units of one dimension, and
``spectral()`` relates energy and length by E lambda = h c.
"""
import math
from contextlib import contextmanager

import numpy as np

_BASE = ('angle', 'length', 'energy', 'time')


class UnitConversionError(Exception):
    pass


class Unit:
    # ndarray * unit -> Unit.__rmul__ (numpy defers), as astropy units do
    __array_ufunc__ = None

    def __init__(self, name, kind, scale, dims=None):
        self.name = name
        self.scale = scale
        if dims is None:
            dims = tuple(1 if k == kind else 0 for k in _BASE)
        self.dims = tuple(dims)
        self.kind = kind if kind is not None else self.dims

    def __rmul__(self, other):
        return Quantity(other, self)

    def __mul__(self, other):
        if isinstance(other, Unit):
            return Unit(self.name + '*' + other.name, None, self.scale * other.scale,
                        tuple(a + b for a, b in zip(self.dims, other.dims)))
        return Quantity(other, self)

    def __rtruediv__(self, other):
        return Quantity(other, dimensionless_unscaled / self)

    def __truediv__(self, other):
        if isinstance(other, Unit):
            return Unit(self.name + '/' + other.name, None, self.scale / other.scale,
                        tuple(a - b for a, b in zip(self.dims, other.dims)))
        return NotImplemented

    def __pow__(self, p):
        return Unit(self.name + '**%s' % p, None, self.scale ** p,
                    tuple(a * p for a in self.dims))

    def is_equivalent(self, other):
        return self.dims == other.dims

    def to(self, other, value=1.0, equivalencies=None):
        return Quantity(value, self).to(other, equivalencies=equivalencies).value

    def __repr__(self):
        return 'Unit(%s)' % self.name

    def __eq__(self, other):
        return isinstance(other, Unit) and self.dims == other.dims and self.scale == other.scale

    def __hash__(self):
        return hash((self.dims, self.scale))


rad = Unit('rad', 'angle', 1.0)
deg = Unit('deg', 'angle', math.pi / 180.)
degree = deg
arcmin = Unit('arcmin', 'angle', math.pi / 180. / 60.)
arcsec = Unit('arcsec', 'angle', math.pi / 180. / 3600.)
mm = Unit('mm', 'length', 1.0)
um = Unit('um', 'length', 1e-3)
micrometer = um
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
_ENERGY, _LENGTH = keV.dims, mm.dims
_ZERO = dimensionless_unscaled.dims
_ANGLE = rad.dims

_PRODUCT = {'multiply': 1, 'true_divide': -1, 'divide': -1}
_SAME_UNIT = {'add', 'subtract', 'maximum', 'minimum', 'fmax', 'fmin', 'clip', 'hypot',
              'remainder', 'mod', 'fmod'}
_COMPARE = {'less', 'less_equal', 'greater', 'greater_equal', 'equal', 'not_equal'}
_KEEP = {'negative', 'positive', 'absolute', 'fabs', 'floor', 'ceil', 'rint', 'trunc',
         'conjugate', 'copysign'}
_DIMLESS_IN = {'exp', 'expm1', 'exp2', 'log', 'log2', 'log10', 'log1p', 'sinh', 'cosh', 'tanh'}
_INVERSE_TRIG = {'arcsin', 'arccos', 'arctan', 'arcsinh', 'arccosh', 'arctanh'}
_TRIG = {'sin', 'cos', 'tan'}


def _split(x):
    if isinstance(x, Quantity):
        return x.view(np.ndarray), x.unit
    return x, None


def _as(v, u, target):
    """Value v in unit u expressed in unit target (same dimension)."""
    if u is None or target is None or u.scale == target.scale:
        return v
    if u.dims != target.dims:
        raise UnitConversionError('%s -> %s' % (u, target))
    return v * (u.scale / target.scale)


def _dimless(v, u):
    """Value of a dimensionless (or plain) operand."""
    if u is None:
        return v
    if u.dims != _ZERO:
        raise UnitConversionError('%s is not dimensionless' % u)
    return v if u.scale == 1.0 else v * u.scale


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

    def __array_ufunc__(self, ufunc, method, *inputs, **kwargs):
        name = ufunc.__name__
        split = [_split(x) for x in inputs]
        vals = [v for v, _ in split]
        units = [u for _, u in split]
        if kwargs.get('out') is not None:
            kwargs['out'] = tuple(o.view(np.ndarray) if isinstance(o, Quantity) else o
                                  for o in kwargs['out'])
        if method == 'reduce' and name in ('add', 'maximum', 'minimum'):
            return Quantity(getattr(ufunc, method)(vals[0], **kwargs), units[0])
        if method != '__call__':
            return getattr(ufunc, method)(*vals, **kwargs)
        first = next(u for u in units if u is not None)
        if name in _PRODUCT and len(vals) == 2:
            ua = units[0] or dimensionless_unscaled
            ub = units[1] or dimensionless_unscaled
            unit = ua * ub if _PRODUCT[name] > 0 else ua / ub
            return Quantity(ufunc(*vals, **kwargs), unit)
        if name in ('power', 'float_power'):
            base = units[0] or dimensionless_unscaled
            if base.dims == _ZERO:       # any exponent, dimensionless result
                return Quantity(ufunc(_dimless(vals[0], units[0]), _dimless(vals[1], units[1]),
                                      **kwargs), dimensionless_unscaled)
            p = float(np.asarray(vals[1]))
            return Quantity(ufunc(*vals, **kwargs), base ** p)
        if name in ('sqrt', 'square', 'cbrt', 'reciprocal'):
            p = {'sqrt': 0.5, 'square': 2, 'cbrt': 1. / 3, 'reciprocal': -1}[name]
            return Quantity(ufunc(*vals, **kwargs), units[0] ** p)
        if name in _SAME_UNIT or name in _COMPARE:
            target = units[0] if units[0] is not None else first
            conv = [_as(v, u, target) for v, u in zip(vals, units)]
            out = ufunc(*conv, **kwargs)
            return out if name in _COMPARE else Quantity(out, target)
        if name in _KEEP:
            return Quantity(ufunc(*vals, **kwargs), first)
        if name in _DIMLESS_IN:
            return Quantity(ufunc(*[_dimless(v, u) for v, u in zip(vals, units)], **kwargs),
                            dimensionless_unscaled)
        if name in _INVERSE_TRIG:
            return Quantity(ufunc(*[_dimless(v, u) for v, u in zip(vals, units)], **kwargs), rad)
        if name == 'arctan2':
            conv = [_as(v, u, first) for v, u in zip(vals, units)]
            return Quantity(ufunc(*conv, **kwargs), rad)
        if name in _TRIG:
            v, u = vals[0], units[0]
            if u is not None and u.dims == _ANGLE:
                v = _as(v, u, rad)
            else:
                v = _dimless(v, u)
            return Quantity(ufunc(v, **kwargs), dimensionless_unscaled)
        return ufunc(*vals, **kwargs)

    @property
    def value(self):
        v = self.view(np.ndarray)
        return v[()] if v.ndim == 0 else v

    def to(self, other, equivalencies=None):
        if self.unit.dims == other.dims:
            if self.unit.scale == other.scale:
                return Quantity(self.value, other)
            return Quantity(self.value * (self.unit.scale / other.scale), other)
        if equivalencies is not None:
            dims = {self.unit.dims, other.dims}
            if dims == {_ENERGY, _LENGTH}:
                # E [keV] * lambda [nm] = hc
                v = self.value * self.unit.scale
                out = _HC_KEV_NM / v
                return Quantity(out * (nm.scale / other.scale), other)
        raise UnitConversionError('%s -> %s' % (self.unit, other))

    def to_value(self, unit=None, equivalencies=None):
        return self.value if unit is None else self.to(unit, equivalencies).value

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
