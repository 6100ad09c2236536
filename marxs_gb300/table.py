"""Columnar photon list with the astropy ``Table`` access pattern.

``PhotonTable`` is what this package hands back when the caller passes a
plain dict; an ``astropy.table.Table`` (or anything with ``colnames``,
``__getitem__``/``__setitem__`` by column name and ``len``) works the same
way with ``GpuSequence``.  Vector columns are ``(N, 4)`` float64 homogeneous
coordinates: ``pos`` (w=1), ``dir`` and ``polarization`` (w=0).
"""
from collections import OrderedDict
import copy as _copy

import numpy as np


class PhotonTable:
    def __init__(self, data=None, meta=None):
        self.columns = OrderedDict()
        self.meta = OrderedDict(meta or {})
        if data is not None:
            items = data.items() if hasattr(data, 'items') else (
                (k, data[k]) for k in data.colnames)
            for k, v in items:
                self[k] = v

    @property
    def colnames(self):
        return list(self.columns.keys())

    def keys(self):
        return self.colnames

    def __len__(self):
        return len(next(iter(self.columns.values()))) if self.columns else 0

    def __contains__(self, key):
        return key in self.columns

    def __getitem__(self, key):
        if isinstance(key, str):
            return self.columns[key]
        out = PhotonTable(meta=_copy.deepcopy(self.meta))
        for k, v in self.columns.items():
            out.columns[k] = np.asarray(v)[key]
        return out

    def __setitem__(self, key, value):
        arr = np.asarray(value)
        if arr.ndim == 0 and self.columns:
            arr = np.full(len(self), arr[()])
        self.columns[key] = np.array(arr, copy=True)

    def add_column(self, col, name=None):
        name = name or getattr(col, 'name')
        self[name] = col

    def remove_column(self, name):
        del self.columns[name]

    def copy(self):
        out = PhotonTable(meta=_copy.deepcopy(self.meta))
        for k, v in self.columns.items():
            out.columns[k] = np.array(v, copy=True)
        return out

    def as_dict(self):
        return {k: v for k, v in self.columns.items()}
