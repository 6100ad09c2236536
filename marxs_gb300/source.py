"""Photons generated on the GPU: a point source seen through a CircleAperture.

``DeviceSource(aperture, energy, polarization, direction)`` replaces the
host chain Source.generate_photons -> FixedPointing -> CircleAperture
(marxs/source/basesources.py:179-260, marxs/optics/aperture.py:39-146) for
the common case of one point source: ``generate(n)`` writes the photons
straight into device columns (``DevicePhotons``), ready for
``GpuSequence.trace_device``, so no photon list crosses the PCIe/C2C link.

* ``aperture``: this package's ``CircleAperture`` or MARXS's (the geometry's
  centre, v_y, v_z, e_x, ``r_inner`` and ``phi`` are read).
* ``energy``: keV (float), a ``RandomArbitraryPdf`` (this package's or
  MARXS's), or a table with columns ``energy`` and ``fluxdensity`` turned
  into one as Source.generate_energies does (basesources.py:190-196).
* ``polarization``: None (unpolarized: uniform angle in [0, 2 pi)) or an angle
  in rad.
* ``direction``: unit direction of travel (default -x, an on-axis source).
* ``precision``: 'fp64' (float64 arithmetic; with pre-drawn uniforms the
  columns equal the reference's to rounding) or 'fp32local' (Philox only:
  the same distributions with float32 trigonometry and integer bin
  thresholds; positions, energies exact to float-float, ~1e-14, the
  aperture offsets and polarization to float32).
"""
import ctypes as C
import math

import numpy as np
import torch

from . import _abi
from .optics import Geometry


class RandomArbitraryPdf:
    """Piecewise-constant pdf sampler with the reference's attributes
    (math/random.py:4-95): ``x`` upper bin edges, ``pdf`` per bin (``pdf[0]``
    ignored), ``bin_width``, ``cdf`` of the (sorted) masses, ``sortindex``."""

    def __init__(self, x, pdf, randomize_in_bin=True, sort=True):
        if not len(x) == len(pdf):
            raise ValueError('x and pdf must have same number of elements.')
        if not np.all(np.array(pdf) >= 0):
            raise ValueError('pdf cannot have negative elements.')
        self.x = np.asarray(x, dtype=float)
        self.bin_width = np.hstack(([0], np.diff(self.x)))
        if not np.all(self.bin_width >= 0):
            raise ValueError('x must be input in increasing order.')
        pdf = np.asarray(pdf, dtype=float) * self.bin_width
        self.sort = sort
        self.randomize_in_bin = randomize_in_bin
        if self.sort:
            self.sortindex = np.argsort(pdf)
            self.pdf = pdf[self.sortindex]
        else:
            self.pdf = pdf
        self.cdf = np.cumsum(self.pdf)


class CircleAperture:
    """Circular (or annular, or sector) entrance aperture (aperture.py:101-146).

    Position keywords as for every element (``position``, ``zoom``,
    ``orientation``, ``pos4d``); ``phi`` = [phi0, phi1] rad, ``r_inner`` in mm.
    """

    def __init__(self, **kwargs):
        phi = kwargs.pop('phi', [0, 2. * np.pi])
        r_inner = kwargs.pop('r_inner', 0.)
        if phi[0] > phi[1]:
            raise ValueError('phi[1] must be greater than phi[0].')
        if (phi[1] - phi[0]) > (2 * np.pi + 1e-6):
            raise ValueError('phi[1] - phi[0] must be less than 2 pi.')
        self.geometry = Geometry(kwargs)
        self.geometry.phi = phi
        self.geometry._geometry['r_inner'] = r_inner
        if r_inner > np.linalg.norm(self.geometry['v_y']):
            raise ValueError('r_inner must be less than size of full aperture.')
        if not np.isclose(np.linalg.norm(self.geometry['v_y']),
                          np.linalg.norm(self.geometry['v_z'])):
            raise ValueError('Aperture does not have the same size in y, z direction.')


def _energy_table(energy):
    """(n_bins, constant, x, width, cdf, sortindex-or-None, randomize_in_bin)."""
    if hasattr(energy, 'cdf') and hasattr(energy, 'bin_width'):
        pdf = energy
    elif hasattr(energy, 'colnames') or isinstance(energy, dict):
        x = np.asarray(energy['energy'], dtype=float)
        y = np.hstack(([0], np.asarray(energy['fluxdensity'], dtype=float)[1:]))
        pdf = RandomArbitraryPdf(x, y)
    else:
        return 0, float(energy), None
    return len(pdf.x), 0.0, pdf


class DeviceSource:
    def __init__(self, aperture, energy=1.0, polarization=None, direction=(-1., 0., 0.),
                 device=None, precision='fp64'):
        if precision not in ('fp64', 'fp32local'):
            raise ValueError("precision must be 'fp64' or 'fp32local'")
        self.precision = precision
        self.device = torch.device('cuda', torch.cuda.current_device()) if device is None \
            else torch.device(device)
        g = aperture.geometry
        self.center = np.asarray(g['center'], dtype=float)[:3]
        self.v_y = np.asarray(g['v_y'], dtype=float)[:3]
        self.v_z = np.asarray(g['v_z'], dtype=float)[:3]
        self.e_x = np.asarray(g['e_x'], dtype=float)[:3]
        self.phi = [float(g.phi[0]), float(g.phi[1])]
        self.r_inner_norm = float(g['r_inner']) / float(np.linalg.norm(np.r_[self.v_y, 0.]))
        d = np.asarray(direction, dtype=float)[:3]
        self.direction = d / np.linalg.norm(d)
        self.polarization = polarization
        self.n_bins, self.energy_value, self.pdf = _energy_table(energy)
        self._tables = None
        # polarization_vectors basis (polarization.py:49-60)
        r = self.direction
        x, y = np.array([1., 0., 0.]), np.array([0., 1., 0.])
        v1 = (x - r * np.dot(r, x)) if (np.isclose(r[0], 0.) and np.isclose(r[2], 0.)) \
            else (y - r * np.dot(r, y))
        self.v1 = v1 / np.linalg.norm(v1)
        self.v2 = np.cross(r, self.v1)
        d4 = np.r_[self.direction, 0.]
        self.prob = float(np.clip(np.dot(d4, -np.r_[self.e_x, 0.]), 0, 1))

    def _device_tables(self):
        if self._tables is None and self.pdf is not None:
            p = self.pdf
            x = np.asarray(p.x, dtype=float)
            w = np.asarray(p.bin_width, dtype=float)
            if not getattr(p, 'randomize_in_bin', True):
                # x[index] instead of x[index - 1] + width * u
                x = np.roll(x, -1)
                w = np.zeros_like(w)
            idx = np.asarray(p.sortindex if getattr(p, 'sort', True) else np.arange(len(x)),
                             dtype=np.int32)
            cdf = np.asarray(p.cdf, dtype=float)
            # float32-local tables: the bin's energy at u = 0 (x[index - 1],
            # numpy's x[-1] wrap included) as float-float, widths as float32,
            # and 32-bit thresholds of the normalised cumulative masses
            lo = np.roll(x, 1) if getattr(p, 'randomize_in_bin', True) else x
            hi32 = lo.astype(np.float32)
            lo32 = (lo - hi32.astype(np.float64)).astype(np.float32)
            thresh = np.minimum(np.floor(cdf / cdf[-1] * 2.0 ** 32) + 1, 2.0 ** 32)
            tabs32 = [np.ascontiguousarray(np.stack([hi32, lo32], axis=1).ravel()),
                      w.astype(np.float32), thresh.astype(np.uint64).view(np.int64)]
            self._tables = [torch.from_numpy(np.ascontiguousarray(a)).to(self.device)
                            for a in [x, w, cdf, idx] + tabs32]
        return self._tables

    def abi(self, n, seed=0, row_base=0, draws=None):
        S = _abi.MgpuSource()
        S.n, S.seed, S.row_base = int(n), int(seed), int(row_base)
        S.rng = _abi.RNG_PREDRAWN if draws is not None else _abi.RNG_PHILOX
        S.n_bins = self.n_bins
        S.energy = self.energy_value
        tabs = self._device_tables()
        if tabs is not None:
            (S.e_x, S.e_width, S.e_cdf, S.e_index, S.e_lo_ff, S.e_width_f,
             S.e_thresh) = [t.data_ptr() for t in tabs]
        S.precision = _abi.FP64 if self.precision == 'fp64' else _abi.FP32LOCAL
        S.pol_random = 1 if self.polarization is None else 0
        S.pol_angle = 0.0 if self.polarization is None else float(self.polarization)
        for name, v in (('dir', self.direction), ('pol_v1', self.v1), ('pol_v2', self.v2),
                        ('center', self.center), ('v_y', self.v_y), ('v_z', self.v_z)):
            getattr(S, name)[:] = [float(a) for a in v]
        S.phi0, S.phi1 = self.phi
        S.r_inner2 = self.r_inner_norm ** 2
        S.prob = self.prob
        if draws is not None:
            S.draws = draws.data_ptr()
        return S

    def generate(self, n, seed=0, row_base=0, draws=None, out=None, stream=None):
        """n photons into ``out`` (DevicePhotons, allocated if None).  ``draws``:
        optional (5, n) float64 device tensor of uniforms (energy choice,
        in-bin, polarization angle, phi, r) instead of Philox."""
        from .gpu import DevicePhotons
        if draws is not None and self.precision != 'fp64':
            raise ValueError('pre-drawn uniforms need precision="fp64"')
        out = DevicePhotons(n, self.device) if out is None else out
        if draws is not None:
            draws = torch.as_tensor(draws, dtype=torch.float64, device=self.device).contiguous()
            if tuple(draws.shape) != (5, n):
                raise ValueError('draws must have shape (5, n)')
        S = self.abi(n, seed, row_base, draws)
        s = torch.cuda.current_stream() if stream is None else stream
        pos, dirs, pol, en, pr = out.abi()
        lib = _abi.load()
        _abi.check(lib.mgpu_generate_photons(C.byref(S), pos, dirs, pol, en, pr,
                                             C.c_void_p(s.cuda_stream)), 'mgpu_generate_photons')
        return out


def simulate_events(source, seq, n, columns=('det_phi', 'det_y', 'order', 'facet'), seed=0,
                    row_base=0, chunk=8_000_000, out=None):
    """Generate ``n`` photons on the GPU, trace them through ``seq`` and
    return the detector event ``columns`` in pinned host memory.

    The photons are processed in chunks alternating over two streams: while
    one chunk is generated and traced, the previous chunk's event columns
    travel to the host, so the host link (the limit for the event list) is
    busy while the GPU computes.  Photon ``k`` of the list gets global id
    ``row_base + k`` whatever the chunking, so the result does not depend on
    ``chunk``.  ``out``: optional dict of pinned host tensors to fill.
    """
    from .gpu import DevicePhotons
    dev = source.device
    chunk = max(1, min(int(chunk), int(n)))
    inst = seq.lower()
    streams = [torch.cuda.Stream(device=dev), torch.cuda.Stream(device=dev)]
    slots = []
    for s in streams:
        with torch.cuda.stream(s):
            plan, bufs = seq.allocate_columns(chunk)
            slots.append({'ph': DevicePhotons(chunk, dev), 'plan': plan, 'bufs': bufs,
                          'status': torch.zeros(1, dtype=torch.int32, device=dev),
                          'hits': torch.zeros(_abi.MAX_STAGES, dtype=torch.int64, device=dev)})
    missing = [c for c in columns if c not in slots[0]['bufs']]
    if missing:
        raise ValueError('the chain writes no column %s' % missing)
    if out is None:
        out = {c: torch.empty(n, dtype=slots[0]['bufs'][c].dtype, pin_memory=True)
               for c in columns}
    cur = torch.cuda.current_stream(dev)
    for s in streams:
        s.wait_stream(cur)
    for k, start in enumerate(range(0, n, chunk)):
        m = min(chunk, n - start)
        sl = slots[k % 2]
        s = streams[k % 2]
        with torch.cuda.stream(s):
            # this slot's buffers are reused only on stream s, after its last copy
            ph = sl['ph'] if m == chunk else _view(sl['ph'], m)
            source.generate(m, seed=seed, row_base=row_base + start, out=ph, stream=s)
            seq.trace_device(ph, ph, sl['plan'], {c: b[:m] for c, b in sl['bufs'].items()},
                             stream=s, status=sl['status'], hits=sl['hits'],
                             row_base=row_base + start, lowered=inst)
            for c in columns:
                out[c][start:start + m].copy_(sl['bufs'][c][:m], non_blocking=True)
    for s in streams:
        cur.wait_stream(s)
    torch.cuda.synchronize(dev)
    for sl in slots:
        code = int(sl['status'].item())
        if code:
            seq._raise_status(code)
    return out


def _view(ph, m):
    """The first m photons of a DevicePhotons (views, no copy)."""
    from .gpu import DevicePhotons
    v = DevicePhotons.__new__(DevicePhotons)
    v.n = m
    v.pos, v.dir, v.pol = ph.pos[:, :m], ph.dir[:, :m], ph.pol[:, :m]
    v.energy, v.prob = ph.energy[:m], ph.prob[:m]
    return v
