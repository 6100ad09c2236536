"""Columnar table with numpy-array columns (the subset the raytrace uses).

``Table[name]`` returns a ``Column`` (ndarray subclass), so masked in-place
assignment such as ``photons['pos'][mask] = value`` modifies the table.
Assigning ``Table[name] = value`` replaces (or adds) the whole column,
broadcasting scalars to the table length.
"""
from collections import OrderedDict
import copy as _copy

import numpy as np


class Column(np.ndarray):
    def __new__(cls, data=None, name=None, dtype=None, shape=(), length=0,
                unit=None, description=None, meta=None, format=None, copy=True):
        if data is None:
            dt = np.dtype(float if dtype is None else dtype)
            arr = np.zeros((length,) + tuple(shape), dtype=dt)
        else:
            arr = np.array(np.asarray(data), dtype=dtype, copy=True)
        obj = arr.view(cls)
        obj.name = name
        obj.unit = unit
        return obj

    def __array_finalize__(self, obj):
        self.name = getattr(obj, 'name', None)
        self.unit = getattr(obj, 'unit', None)

    @property
    def data(self):
        return self.view(np.ndarray)

    @property
    def value(self):
        return self.view(np.ndarray)

    def to(self, unit, equivalencies=None):
        from astropy.units import Quantity
        return Quantity(self.view(np.ndarray), self.unit).to(unit, equivalencies=equivalencies)


MaskedColumn = Column


class TableColumns(OrderedDict):
    """Columns by name, by position, or a slice of positions."""

    def __getitem__(self, key):
        if isinstance(key, (int, np.integer)):
            return list(self.values())[key]
        if isinstance(key, slice):
            return TableColumns(list(self.items())[key])
        return OrderedDict.__getitem__(self, key)


class Row:
    def __init__(self, table, index):
        self._table = table
        self.index = index

    def __getitem__(self, key):
        return self._table.columns[key][self.index]

    @property
    def colnames(self):
        return self._table.colnames


class Table:
    def __init__(self, data=None, names=None, meta=None, masked=None, copy=True,
                 dtype=None, rows=None):
        self.columns = TableColumns()
        self.meta = OrderedDict(meta or {})
        if data is None:
            return
        if isinstance(data, Table):
            for k in data.colnames:
                self[k] = data[k]
            self.meta = _copy.deepcopy(data.meta)
        elif isinstance(data, dict):
            for k, v in data.items():
                self[k] = v
        else:
            for i, col in enumerate(data):
                name = names[i] if names is not None else getattr(col, 'name', 'col%d' % i)
                self[name] = col
                if getattr(col, 'unit', None) is not None:
                    self.columns[name].unit = col.unit

    @property
    def colnames(self):
        return list(self.columns.keys())

    def keys(self):
        return self.colnames

    def __len__(self):
        if not self.columns:
            return 0
        return len(next(iter(self.columns.values())))

    def __contains__(self, key):
        return key in self.columns

    def _as_column(self, name, value):
        unit = getattr(value, 'unit', None)
        arr = np.asarray(value)
        if arr.ndim == 0 and len(self.columns) > 0:
            arr = np.full(len(self), arr[()])
        col = Column(arr, name=name)
        col.unit = unit
        return col

    def __getitem__(self, key):
        if isinstance(key, str):
            return self.columns[key]
        if isinstance(key, (int, np.integer)):
            return Row(self, key)
        out = Table(meta=_copy.deepcopy(self.meta))
        for k, v in self.columns.items():
            out.columns[k] = Column(np.asarray(v)[key], name=k)
        return out

    def __setitem__(self, key, value):
        if isinstance(key, str):
            self.columns[key] = self._as_column(key, value)
        else:
            raise NotImplementedError('row assignment not supported by the shim')

    def add_column(self, col, name=None, index=None, copy=True):
        name = name or col.name
        if not isinstance(col, Column):
            # copy=False keeps the caller's array (a view, no copy), as astropy
            col = self._as_column(name, col) if copy else np.asarray(col).view(Column)
        col.name = name
        self.columns[name] = col

    def remove_column(self, name):
        del self.columns[name]

    def copy(self, copy_data=True):
        out = Table(meta=_copy.deepcopy(self.meta))
        for k, v in self.columns.items():
            c = Column(np.array(v), name=k)
            c.unit = getattr(v, 'unit', None)
            out.columns[k] = c
        return out

    @classmethod
    def read(cls, filename, format=None, **kwargs):
        """ECSV only: '#' header with '- {name: .., unit: ..}' column
        entries, a line of column names, whitespace-separated values."""
        import re
        import astropy.units as u
        if format not in (None, 'ascii.ecsv'):
            raise NotImplementedError('Table.read: only ECSV in the test shim')
        units, names, rows = {}, None, []
        with open(filename) as fh:
            for line in fh:
                if line.startswith('#'):
                    m = re.search(r'name:\s*([^,}]+)', line)
                    if m and 'datatype' in line:
                        un = re.search(r'unit:\s*([^,}]+)', line)
                        units[m.group(1).strip()] = un.group(1).strip() if un else None
                    continue
                if not line.strip():
                    continue
                if names is None:
                    names = line.split()
                    continue
                rows.append([float(v) for v in line.split()])
        data = np.array(rows, dtype=float).reshape(-1, len(names))
        out = cls()
        for j, name in enumerate(names):
            out[name] = data[:, j]
            un = units.get(name)
            if un is not None:
                out.columns[name].unit = getattr(u, un)
        return out


QTable = Table


def join(*args, **kwargs):
    raise NotImplementedError('join is not provided by the test shim')


def vstack(tables, **kwargs):
    out = Table()
    for k in tables[0].colnames:
        out[k] = np.concatenate([np.asarray(t[k]) for t in tables])
    return out
