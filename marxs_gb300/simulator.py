"""Containers mirroring ``marxs.simulator``: ``Sequence``, ``Parallel`` and
``ParallelCalculated``.

``Parallel.generate_elements`` restates the FP64 pose composition of
marxs/simulator/simulator.py:384-440 (11-matrix chain, :424-437): global
pose, global uncertainty, per-element uncertainty translation, element
centre, common offset, per-element uncertainty rotation, element rotation,
common rotation, uncertainty zoom, element zoom, common zoom.
"""
import numpy as np

from .geomath import (parse_position_keywords, decompose44, translation2aff,
                      mat2aff, zoom2aff, compose, e2h, h2e)
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


def _normalized(vec):
    # transforms3d.utils.normalized_vector: vec / sqrt(sum(vec ** 2))
    vec = np.asarray(vec, dtype=float)
    return vec / np.sqrt(np.sum(vec * vec))


def _ex2vec_fix(e1, efix):
    """Rotation taking x to ``e1`` with the new y coplanar with ``efix``
    (marxs/math/rotations.py:8-47, vectors normalised as transforms3d does)."""
    e1 = _normalized(e1)
    efix = _normalized(efix)
    if np.allclose(e1, efix) or np.allclose(e1, -efix):
        raise ValueError('Input vectors are parallel - Rotation matrix is ambiguous.')
    rot = np.empty((3, 3))
    rot[:, 0] = e1
    rot[:, 1] = _normalized(efix - np.dot(efix, e1) * e1)
    rot[:, 2] = np.cross(rot[:, 0], rot[:, 1])
    return rot


class ParallelCalculated(Parallel):
    """Parallel whose element poses are computed from three specifications
    (marxs/simulator/simulator.py:443-541): ``pos_spec`` the centres
    ((n, 4) homogeneous points, or a callable returning them),
    ``normal_spec`` the element normals (a homogeneous direction shared by
    all, a point they all face away from, or a callable of the centres) and
    ``parallel_spec`` a direction one element side stays parallel to (same
    forms; a callable gets the centres and the normals).  Element i is posed
    as compose(centre_i, ex2vec_fix(normal_i, parallel_i), 1).
    """

    def __init__(self, **kwargs):
        self.pos_spec = kwargs.pop('pos_spec')
        self.normal_spec = kwargs.pop('normal_spec')
        self.parallel_spec = kwargs.pop('parallel_spec')
        kwargs['elem_pos'] = self.calculate_elempos()
        super().__init__(**kwargs)

    def calculate_elempos(self):
        xyzw = self.get_elemxyzw()
        normals = self.get_spec('normal_spec', xyzw)
        parallels = self.get_spec('parallel_spec', xyzw, normals)
        return [compose(h2e(xyzw[i, :]), _ex2vec_fix(h2e(normals[i, :]), h2e(parallels[i, :])),
                        np.ones(3)) for i in range(xyzw.shape[0])]

    def get_elemxyzw(self):
        return self.pos_spec() if callable(self.pos_spec) else self.pos_spec

    def get_spec(self, specname, xyzw, *args, **kwargs):
        spec = getattr(self, specname)
        if callable(spec):
            return spec(xyzw, *args, **kwargs)
        if len(spec) == 4:
            if spec[3] == 0:          # a direction shared by all elements
                return np.tile(spec, (xyzw.shape[0], 1))
            return e2h(h2e(xyzw) - h2e(spec)[None, :], 1)   # away from a point
        raise ValueError(specname + 'must be callable or homogeneous coordinate.')
