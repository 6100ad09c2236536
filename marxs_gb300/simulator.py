"""Containers mirroring ``marxs.simulator``: ``Sequence`` and ``Parallel``.

``Parallel.generate_elements`` restates the FP64 pose composition of
marxs/simulator/simulator.py:384-440 (11-matrix chain, :424-437): global
pose, global uncertainty, per-element uncertainty translation, element
centre, common offset, per-element uncertainty rotation, element rotation,
common rotation, uncertainty zoom, element zoom, common zoom.
"""
import numpy as np

from .geomath import (parse_position_keywords, decompose44, translation2aff,
                      mat2aff, zoom2aff)
from .optics import BaseContainer, FinitePlane, Geometry


class SimulationSetupError(Exception):
    pass


class Sequence(BaseContainer):
    """Ordered chain of elements (marxs/simulator/simulator.py:145-203)."""

    def __init__(self, **kwargs):
        self.elements = kwargs.pop('elements')
        super().__init__(**kwargs)

    def __call__(self, photons):
        from .gpu import GpuSequence
        return GpuSequence(elements=self.elements)(photons)


class Parallel(BaseContainer):
    """Group of similar elements of which each photon meets at most one.

    The GPU backend lowers the group to a facet table and finds, per photon,
    the nearest facet it intersects (uniform-grid lookup); MARXS applies the
    facets one after the other (simulator.py:42-49, 209-212).  Both agree
    whenever a ray crosses at most one facet.
    """
    id_col = 'element'
    uncertainty = np.eye(4)

    def __init__(self, **kwargs):
        geometry = kwargs.pop('geometry', FinitePlane)
        if isinstance(geometry, Geometry):
            self.geometry = geometry
        else:
            self.geometry = geometry(kwargs)
        self.id_num_offset = kwargs.pop('id_num_offset', 0)
        self.elem_class = kwargs.pop('elem_class')
        self.elem_args = kwargs.pop('elem_args', {}).copy()
        elem_pos = kwargs.pop('elem_pos')
        if isinstance(elem_pos, dict):
            keys = list(elem_pos.keys())
            for i in range(len(keys) - 1):
                if (not hasattr(elem_pos[keys[i]], '__len__') or
                        not hasattr(elem_pos[keys[i + 1]], '__len__') or
                        len(elem_pos[keys[i]]) != len(elem_pos[keys[i + 1]])):
                    raise ValueError('All elements in elem_pos must have the same number of entries.')
            n = len(elem_pos[keys[0]])
            self.elem_pos = [parse_position_keywords({k: elem_pos[k][i] for k in keys})
                             for i in range(n)]
        else:
            self.elem_pos = [np.asarray(p, dtype=float) for p in elem_pos]
        super().__init__(**kwargs)
        if 'id_col' not in self.elem_args:
            self.elem_args['id_col'] = self.id_col
        self.elem_uncertainty = [np.eye(4)] * len(self.elem_pos)
        self.generate_elements()

    @property
    def pos4d(self):
        return self.geometry.pos4d

    def __call__(self, photons):
        from .gpu import GpuSequence
        return GpuSequence(elements=[self])(photons)

    def generate_elements(self):
        self.elements = []
        for i in range(len(self.elem_pos)):
            args = self.elem_args.copy()
            specific = {}
            for k, v in args.items():
                if isinstance(v, list) and (len(v) == len(self.elem_pos)):
                    specific[k] = v[i]
                else:
                    specific[k] = v
            if 'name' not in specific:
                specific['name'] = 'Elem {0} in {1}'.format(i, self.name)
            elem_pos4d = parse_position_keywords(specific)
            telem, relem, zelem, Selem = decompose44(elem_pos4d)
            if not np.allclose(Selem, 0.):
                raise ValueError('pos4 for elem includes shear, which is not supported here.')
            e_center, e_rot, e_zoom, _ = decompose44(self.elem_pos[i])
            tsig, rsig, zsig, ssig = decompose44(self.elem_uncertainty[i])
            if not np.allclose(ssig, 0.):
                raise SimulationSetupError('Shear is not supported in the elem uncertainty.')
            f_pos4d = np.eye(4)
            for m in reversed([self.pos4d, self.uncertainty,
                               translation2aff(tsig), translation2aff(e_center),
                               translation2aff(telem), mat2aff(rsig), mat2aff(e_rot),
                               mat2aff(relem), zoom2aff(zsig), zoom2aff(e_zoom),
                               zoom2aff(zelem)]):
                f_pos4d = np.dot(m, f_pos4d)
            self.elements.append(self.elem_class(pos4d=f_pos4d, id_num=self.id_num_offset + i,
                                                 **specific))
