"""Tolerancing on the GPU: facet poses drawn and applied on the device, and
the trace and analysis of every parameter set run without the photon list
leaving the device.

Mirrors marxs/design/tolerancing.py for facet arrays:

* ``DeviceFacetPoses(seq, parallel)``: the facets of one Parallel inside a
  GpuSequence, posed on the device (mgpu_facet_poses) as
  Parallel.generate_elements poses them (simulator/simulator.py:384-440),
  with the candidate grid rebuilt on the device after every change;
* ``wiggle`` / ``moveglobal`` / ``moveindividual`` (tolerancing.py:45-111)
  with the reference's arguments, acting on a DeviceFacetPoses (or a list
  of them) instead of the host Parallel; wiggle draws its Gaussian
  uncertainties with Philox on the device (the distribution of
  generate_facet_uncertainty, design/uncertainties.py:8-39);
* ``run_tolerances`` (tolerancing.py:224-283) with the reference's
  arguments and result list; ``photons_in`` is a DevicePhotons (or a photon
  table, uploaded once) and ``analyzefunc`` gets the device event columns
  (e.g. ``analysis.CaptureResAeff``).

The device tables belong to the GpuSequence's lowered instrument: a change
of the host elements that makes the sequence lower again discards them.
"""
import ctypes as C
import math
from collections.abc import Iterable
from copy import copy

import numpy as np
import torch

from . import _abi
from .geomath import compose, decompose44, euler2mat, parse_position_keywords


def local_poses(parallel):
    """Uncertainty-free pose of every element in the Parallel's frame: the
    element centre plus the common offset (3) and the product of the element
    rotation, common rotation and zooms (3x3, row-major), as
    Parallel.generate_elements composes them."""
    n = len(parallel.elem_pos)
    out = np.zeros((n, 12))
    for i in range(n):
        specific = {}
        for k, v in parallel.elem_args.items():
            specific[k] = v[i] if (isinstance(v, list) and len(v) == n) else v
        telem, relem, zelem, selem = decompose44(parse_position_keywords(specific))
        if not np.allclose(selem, 0.):
            raise ValueError('pos4 for elem includes shear, which is not supported here.')
        e_center, e_rot, e_zoom, _ = decompose44(np.asarray(parallel.elem_pos[i], dtype=float))
        M = e_rot @ relem @ np.diag(e_zoom) @ np.diag(zelem)
        out[i, :3] = e_center + telem
        out[i, 3:] = M.ravel()
    return out


def _six(dx, dy, dz, rx, ry, rz):
    return [float(dx), float(dy), float(dz), float(rx), float(ry), float(rz)]


class DeviceFacetPoses:
    """Device-side poses of the facets of ``parallel`` inside ``seq``.

    ``max_shift`` (mm) widens the candidate grid so that facets may move by
    up to about that much; a facet that leaves the grid raises on the next
    update.  Each ``wiggle`` without a seed draws a new realisation.
    """

    def __init__(self, seq, parallel, max_shift=10.0, seed=0):
        self.seq = seq
        self.parallel = parallel
        self.inst = seq.lower()
        stages = [k for k, st in enumerate(self.inst.stages)
                  if st.kind == _abi.STAGE_GRATINGS and st.element is parallel]
        if len(stages) != 1:
            raise ValueError('the sequence has no facet stage for this Parallel')
        self.si = si = stages[0]
        st = self.inst.stages[si]
        self.n = len(st.facets)
        if self.n != len(parallel.elem_pos):
            raise ValueError('facet table and Parallel differ in size')
        dev = self.inst.device
        self.device = dev
        groove = np.array([float(g.geometry._geometry.get('groove_angle', 0.))
                           for g in parallel.elements])
        gs = np.empty((self.n, 2))
        for gv in np.unique(groove):
            k = groove == gv
            gs[k, 0] = math.sin(-gv)
            gs[k, 1] = math.cos(-gv)
        self.local = torch.from_numpy(local_poses(parallel)).to(dev)
        self.groove = torch.from_numpy(gs).to(dev)
        self.perturbation = torch.zeros((self.n, 6), dtype=torch.float64, device=dev)
        self.uncertainty = np.asarray(parallel.uncertainty, dtype=float)
        self.seed = int(seed)
        self._draws = 0
        self._status = torch.zeros(1, dtype=torch.int32, device=dev)
        self._grid(max_shift)

    # ---------------------------------------------------------------- grid
    def _grid(self, pad):
        """Replace the stage's candidate grid by one padded by ``pad`` mm on
        every side, with twice the entry capacity."""
        st = self.inst.stages[self.si]
        if st.grid is None:
            self._rebuild_fn = None
            return
        g = dict(st.grid)
        extra = int(math.ceil(pad / g['cell']))
        g['u0'] -= extra * g['cell']
        g['v0'] -= extra * g['cell']
        g['nu'] += 2 * extra
        g['nv'] += 2 * extra
        g['capacity'] = 2 * g['capacity'] + 64
        stream = torch.cuda.current_stream(self.device)
        self._rebuild_fn = self.inst.set_grid(self.si, g, self._status,
                                              C.c_void_p(stream.cuda_stream))
        self._check()

    def _rebuild(self, stream):
        if self._rebuild_fn is not None:
            self._rebuild_fn(C.c_void_p(stream.cuda_stream))

    def _check(self):
        code = int(self._status.item())
        if code & (_abi.STATUS_GRID_RANGE | _abi.STATUS_GRID_FULL):
            self._status.zero_()
            raise RuntimeError('facets moved outside the candidate grid (status 0x%x): create '
                               'DeviceFacetPoses with a larger max_shift' % code)

    # ---------------------------------------------------------------- poses
    def _apply(self, mode, sigma=(0,) * 6, offset=(0,) * 6, given=None, seed=0):
        dev = self.device
        U = _abi.MgpuPoseUpdate()
        U.n_facets = self.n
        U.mode = mode
        U.seed = int(seed) & 0xffffffffffffffff
        U.sigma[:] = [float(x) for x in sigma]
        U.offset[:] = [float(x) for x in offset]
        if given is not None:
            given = torch.as_tensor(given, dtype=torch.float64, device=dev).contiguous()
            if tuple(given.shape) != (self.n, 6):
                raise ValueError('given perturbations must have shape (%d, 6)' % self.n)
            U.given = given.data_ptr()
        out = torch.empty((self.n, 6), dtype=torch.float64, device=dev)
        U.perturb_out = out.data_ptr()
        outer = np.asarray(self.parallel.pos4d, dtype=float) @ self.uncertainty
        U.outer[:] = [float(x) for x in outer.ravel()]
        U.local = self.local.data_ptr()
        U.groove = self.groove.data_ptr()
        U.facets = self.inst.stage_facets[self.si].data_ptr()
        if self.si in self.inst.stage_facets32:
            U.facets32 = self.inst.stage_facets32[self.si].data_ptr()
        stream = torch.cuda.current_stream(dev)
        lib = _abi.load()
        _abi.check(lib.mgpu_facet_poses(C.byref(U), C.c_void_p(stream.cuda_stream)),
                   'mgpu_facet_poses')
        self._rebuild(stream)
        self.perturbation = out
        self._check()
        return out

    def wiggle(self, dx=0, dy=0, dz=0, rx=0., ry=0., rz=0., seed=None):
        """New Gaussian element uncertainties: sigma dx, dy, dz (mm), rx, ry, rz (rad)."""
        if seed is None:
            seed = (self.seed << 20) + self._draws
            self._draws += 1
        return self._apply(_abi.POSE_DRAW, sigma=_six(dx, dy, dz, rx, ry, rz), seed=seed)

    def moveindividual(self, dx=0, dy=0, dz=0, rx=0, ry=0, rz=0):
        """The same translation and rotation for every element."""
        return self._apply(_abi.POSE_DRAW, offset=_six(dx, dy, dz, rx, ry, rz))

    def moveglobal(self, dx=0, dy=0, dz=0, rx=0., ry=0., rz=0.):
        """Global uncertainty of the Parallel; element uncertainties kept."""
        self.uncertainty = compose([dx, dy, dz], euler2mat(rx, ry, rz, 'sxyz'), np.ones(3))
        return self._apply(_abi.POSE_GIVEN, given=self.perturbation.clone())

    def set_perturbation(self, given):
        """Element uncertainties given as (n_facets, 6): dx, dy, dz, rx, ry, rz."""
        return self._apply(_abi.POSE_GIVEN, given=given)

    def reset(self):
        """No element uncertainty, the Parallel's own global uncertainty."""
        self.uncertainty = np.asarray(self.parallel.uncertainty, dtype=float)
        return self._apply(_abi.POSE_ZERO)


def _each(elements):
    return elements if isinstance(elements, Iterable) else [elements]


def wiggle(e, dx=0, dy=0, dz=0, rx=0., ry=0., rz=0.):
    """Move and rotate each facet by Gaussian amounts (sigma per axis)."""
    for x in _each(e):
        x.wiggle(dx, dy, dz, rx, ry, rz)


def moveglobal(e, dx=0, dy=0, dz=0, rx=0., ry=0., rz=0.):
    """Move and rotate the whole Parallel."""
    for x in _each(e):
        x.moveglobal(dx, dy, dz, rx, ry, rz)


def moveindividual(e, dx=0, dy=0, dz=0, rx=0, ry=0, rz=0):
    """Move and rotate every facet by the same amount."""
    for x in _each(e):
        x.moveindividual(dx, dy, dz, rx, ry, rz)


def run_tolerances(photons_in, instrum, wigglefunc, wiggleparts, parameters, analyzefunc):
    """For every parameter dict: ``wigglefunc(wiggleparts, **pars)``, trace
    ``photons_in`` through ``instrum`` (a GpuSequence) on the device, and
    ``analyzefunc(columns)`` on the device event columns (every column the
    chain writes, plus ``probability`` and ``energy``).  Returns one dict
    per parameter set: the parameters updated with the analysis result."""
    from .gpu import DevicePhotons
    if not isinstance(photons_in, DevicePhotons):
        photons_in = DevicePhotons.from_columns(photons_in)
    n = photons_in.n
    plan, bufs = instrum.allocate_columns(n)
    out = DevicePhotons(n, photons_in.pos.device)
    results = []
    for pars in parameters:
        wigglefunc(wiggleparts, **pars)
        status, _ = instrum.trace_device(photons_in, out, plan, bufs)
        code = int(status.item())
        if code:
            instrum._raise_status(code)
        cols = dict(bufs)
        cols['probability'] = out.prob
        cols['energy'] = out.energy
        cpars = copy(pars)
        cpars.update(analyzefunc(cols))
        results.append(cpars)
    return results
