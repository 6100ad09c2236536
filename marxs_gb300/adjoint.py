"""Pose gradients of detector-plane losses through a hand-written adjoint.

The chain is the grating spectrometer the raytrace kernels run:
PerfectLens (optics/mirror.py:53-82) -> RadialMirrorScatter
(optics/scatter.py:49-77) -> a Parallel array of FlatGrating / CATGrating
facets (optics/grating.py:233-277, simulator/simulator.py:206-212) ->
FlatDetector or CircularDetector (math/geometry.py:211-261, 470-564).

A GPU trace decides every photon's discrete choices: which facet it meets,
its order, its scatter angles, its weight (probability), the order sign of
CAT gratings, the side of the facet normal it leaves on and, on a cylinder,
which root of the intersection it takes.  With those frozen, the detector
coordinates are smooth functions of the parameters

    theta = [f, facet_0 (t_x, t_y, t_z, a_x, a_y, a_z), ..., facet_{F-1},
             detector (t_x, t_y, t_z, a_x, a_y, a_z)]

(f the focal length; t a translation of the element centre; a static-frame
x, y, z Euler angles of a rotation about the centre, the convention of
design/uncertainties.py:36-38), and ``mgpu_pose_adjoint`` returns per-group
moments of the detector spot and, in one reverse launch, the gradient of any
loss written over those moments.  ``PoseMoments`` wraps that as a
``torch.autograd.Function``.
"""
import ctypes as C
import math

import numpy as np
import torch

from . import _abi
from .geomath import euler2mat
from .lowering import _grating_facets, classnames, cylinder_block, host_evaluated

FWHM_PER_SIGMA = 2.0 * math.sqrt(2.0 * math.log(2.0))


def _stream_handle(stream=None):
    s = torch.cuda.current_stream() if stream is None else stream
    return C.c_void_p(s.cuda_stream)


def _ptr(t):
    return C.c_void_p(t.data_ptr()) if t is not None else C.c_void_p(0)


def _unit(v):
    v = np.asarray(v, dtype=float)[:3]
    return v / np.linalg.norm(v)


def _chain_parts(elements):
    """(lens, scatter, gratings, detector) of a lens -> scatter -> facets -> detector chain."""
    parts = {}
    for e in elements:
        names = classnames(e)
        if 'PerfectLens' in names:
            parts['lens'] = e
        elif 'RadialMirrorScatter' in names:
            parts['scatter'] = e
        elif 'Parallel' in names:
            parts['gratings'] = (e, list(e.elements))
        elif {'FlatGrating', 'CATGrating'} & names:
            parts['gratings'] = (e, [e])
        elif 'FlatDetector' in names:
            parts['detector'] = (e, _abi.ADJ_DET_FLAT)
        elif 'CircularDetector' in names:
            parts['detector'] = (e, _abi.ADJ_DET_CYL)
        else:
            raise NotImplementedError('pose adjoint: element %s' % type(e).__name__)
    missing = {'lens', 'scatter', 'gratings', 'detector'} - set(parts)
    if missing:
        raise NotImplementedError('pose adjoint needs lens, scatter, gratings and detector; '
                                  'missing %s' % sorted(missing))
    return parts


def euler_sxyz(a):
    """Rz(a2) Ry(a1) Rx(a0) (numpy, host)."""
    return euler2mat(a[0], a[1], a[2], 'sxyz')


def euler_sxyz_batch(a):
    """(F, 3) angles -> (F, 3, 3) matrices Rz(a2) Ry(a1) Rx(a0)."""
    c, s = np.cos(a), np.sin(a)
    F = len(a)
    Rx = np.zeros((F, 3, 3))
    Ry = np.zeros((F, 3, 3))
    Rz = np.zeros((F, 3, 3))
    Rx[:, 0, 0] = 1
    Rx[:, 1, 1], Rx[:, 1, 2], Rx[:, 2, 1], Rx[:, 2, 2] = c[:, 0], -s[:, 0], s[:, 0], c[:, 0]
    Ry[:, 1, 1] = 1
    Ry[:, 0, 0], Ry[:, 0, 2], Ry[:, 2, 0], Ry[:, 2, 2] = c[:, 1], s[:, 1], -s[:, 1], c[:, 1]
    Rz[:, 2, 2] = 1
    Rz[:, 0, 0], Rz[:, 0, 1], Rz[:, 1, 0], Rz[:, 1, 1] = c[:, 2], -s[:, 2], s[:, 2], c[:, 2]
    return Rz @ Ry @ Rx


class PoseModel:
    """Nominal poses of the chain and the map from theta to element poses.

    The facet and detector poses held here are the base every theta is
    applied to: a perturbed element gets pos4d = [R M | c + t] for the base
    pos4d = [M | c]; the lens gets focal length theta[0].
    """

    def __init__(self, elements):
        self.elements = list(elements)
        p = _chain_parts(self.elements)
        self.lens = p['lens']
        self.scatter = p['scatter']
        self.grating_owner, self.gratings = p['gratings']
        self.detector, self.det_kind = p['detector']
        self.n_facets = len(self.gratings)
        if self.n_facets > _abi.ADJ_MAX_FACETS:
            raise NotImplementedError('pose adjoint: more than %d facets' % _abi.ADJ_MAX_FACETS)
        self.n_params = 7 + 6 * self.n_facets
        self.focallength = float(self.lens.focallength)
        self.facet_pos4d = [np.array(g.geometry.pos4d, dtype=float) for g in self.gratings]
        self._base_stack = np.stack(self.facet_pos4d)
        self.det_pos4d = np.array(self.detector.geometry.pos4d, dtype=float)
        self.facet_index = {int(g.id_num): i for i, g in enumerate(self.gratings)}
        self._tables()

    # ------------------------------------------------------------ fixed data
    def _tables(self):
        lp = np.asarray(self.lens.geometry.pos4d, dtype=float)
        self.lens_block = np.concatenate([lp[:3, 3], _unit(lp[:, 0]), _unit(lp[:, 2]),
                                          [float(getattr(self.lens, 'd_center_optax', 0.))]])
        sp = np.asarray(self.scatter.geometry.pos4d, dtype=float)
        self.scatter_block = np.concatenate([sp[:3, 3], _unit(sp[:, 0])])
        hd, hb = host_evaluated(self.gratings)
        if any('Cylinder' in classnames(g.geometry) for g in self.gratings):
            raise NotImplementedError('pose gradients of gratings on Cylinder surfaces')
        if hd or hb:
            raise NotImplementedError('pose gradients of gratings with a position-dependent '
                                      'grating constant or blaze modifier')
        fac = _grating_facets(self.gratings, [], {})
        base = np.empty((self.n_facets, 13))
        base[:, 0:3] = fac['c']
        base[:, 3:6] = fac['ex']
        base[:, 6:9] = fac['l']
        base[:, 9:12] = fac['dneg']
        base[:, 12] = fac['dgrat']
        self.facet_base = base
        self.facet_flags = (fac['cat'].astype(np.uint8) * _abi.ADJ_FACET_CAT |
                            fac['transmission'].astype(np.uint8) * _abi.ADJ_FACET_TRANSMISSION)
        det = np.zeros(32)
        dp = self.det_pos4d
        if self.det_kind == _abi.ADJ_DET_FLAT:
            det[0:3] = dp[:3, 3]
            det[3:6] = _unit(dp[:, 0])
            det[6:9] = _unit(dp[:, 1])
            det[9:12] = _unit(dp[:, 2])
        else:
            cb = cylinder_block(self.detector.geometry)
            M = dp[:3, :3]
            det[0:3] = dp[:3, 3]
            det[3:12] = M.ravel()
            det[12:21] = np.linalg.inv(M).ravel()
            det[21] = cb[25]            # radius (zoom x)
            det[22] = cb[24]            # zoom z
            det[23] = cb[26]            # reduced phi borders
            det[24] = cb[27]
        self.det_block = det

    def theta0(self, device=None):
        th = torch.zeros(self.n_params, dtype=torch.float64, device=device)
        th[0] = self.focallength
        return th

    def param_slices(self):
        F = self.n_facets
        idx = np.arange(self.n_params)
        return {'focal_length': idx[:1],
                'facet_translation': (1 + 6 * np.arange(F)[:, None] + np.arange(3)).ravel(),
                'facet_rotation': (4 + 6 * np.arange(F)[:, None] + np.arange(3)).ravel(),
                'detector_translation': 1 + 6 * F + np.arange(3),
                'detector_rotation': 4 + 6 * F + np.arange(3)}

    def step_sizes(self, h_trans=1e-4, h_rot=1e-6, h_f=1e-4):
        """Central-difference steps: h_trans (mm) for translations and the
        focal length, h_rot (rad) for rotations."""
        h = np.full(self.n_params, h_trans)
        h[0] = h_f
        sl = self.param_slices()
        h[sl['facet_rotation']] = h_rot
        h[sl['detector_rotation']] = h_rot
        return h

    # --------------------------------------------------------- poses <- theta
    def apply(self, theta):
        """Set the element poses (and focal length) for ``theta`` (all facets
        at once: R = Rz Ry Rx per facet, pos4d = [R M | c + t])."""
        th = np.asarray(theta.detach().cpu() if torch.is_tensor(theta) else theta, dtype=float)
        self.lens.focallength = float(th[0])
        F = self.n_facets
        p6 = th[1:1 + 6 * F].reshape(F, 6)
        new = np.array(self._base_stack, copy=True)
        new[:, :3, :3] = euler_sxyz_batch(p6[:, 3:6]) @ self._base_stack[:, :3, :3]
        new[:, :3, 3] += p6[:, 0:3]
        for g, m in zip(self.gratings, new):
            g.geometry.pos4d = m
        self.detector.geometry.pos4d = self._perturbed(self.det_pos4d, th[1 + 6 * F:7 + 6 * F])

    def restore(self):
        self.apply(np.concatenate([[self.focallength], np.zeros(self.n_params - 1)]))

    @staticmethod
    def _perturbed(pos4d, p6):
        out = pos4d.copy()
        R = euler_sxyz(p6[3:6])
        out[:3, :3] = R @ pos4d[:3, :3]
        out[:3, 3] = pos4d[:3, 3] + p6[0:3]
        return out

    # --------------------------------------------------------- frozen photons
    def trace(self, photons, orders, draws=None, precision='fp64', rng=None, seed=0,
              theta=None, energy_range=None, device=None, freeze=True, process_group=None,
              row_base=0, adjoint_precision='fp64'):
        """Trace ``photons`` (host columns or DevicePhotons) through the
        elements as they are posed now and freeze the result.  ``precision``
        is the raytrace's, ``adjoint_precision`` the frozen photons' moments
        and gradients' (``FrozenPhotons.precision``).

        Returns (FrozenPhotons or None if not ``freeze``, trace) with trace =
        (sequence, input, output, column buffers) of the device run.  For
        photons sharded over a process group, ``row_base`` is the global id
        of this rank's first photon (its Philox streams) and the frozen
        photons sum their moments and gradients over ``process_group``.
        """
        from .gpu import DevicePhotons, GpuSequence
        rng = rng or ('predrawn' if draws is not None else 'philox')
        seq = GpuSequence(self.elements, precision=precision, rng=rng, seed=seed, device=device)
        inp = photons if isinstance(photons, DevicePhotons) else \
            DevicePhotons.from_columns(photons, seq.device)
        out = DevicePhotons(inp.n, seq.device)
        plan, bufs = seq.allocate_columns(inp.n)
        status, _ = seq.trace_device(inp, out, plan, bufs, draws=draws, row_base=row_base)
        seq._raise_status(int(status.item()))
        if not freeze:
            return None, (seq, inp, out, bufs)
        frozen = self.freeze_trace(seq, inp, out, bufs, orders, energy_range, theta,
                                   process_group, adjoint_precision)
        return frozen, (seq, inp, out, bufs)

    def freeze_trace(self, seq, inp, out, bufs, orders, energy_range=None, theta=None,
                     process_group=None, adjoint_precision='fp64'):
        """Frozen photons of a device trace ``seq.trace_device(inp, out, ...)``.

        Photons count when they met a facet and the detector; group g holds
        order ``orders[g]`` (and, if given, energies inside energy_range).
        ``theta`` is the parameter vector the traced geometry corresponds to
        (default: nominal).
        """
        st = seq.lower().stages
        names = {s.kind: s for s in st}
        sc = names[_abi.STAGE_SCATTER]
        gr = names[_abi.STAGE_GRATINGS]
        dt = names.get(_abi.STAGE_FLATDET) or names.get(_abi.STAGE_CYLDET)
        alpha, beta = bufs[sc.out_names[2]], bufs[sc.out_names[3]]
        order = bufs[gr.out_names[2]]
        facet_id = bufs[gr.id_col]
        det_loc = bufs[dt.out_names[0]]
        dev = inp.pos.device
        ok = torch.isfinite(det_loc) & (facet_id >= 0) & torch.isfinite(alpha) & \
            torch.isfinite(beta)
        group = torch.full_like(facet_id, -1)
        for g, m in enumerate(orders):
            group = torch.where(ok & (order == float(m)), torch.full_like(group, g), group)
        if energy_range is not None:
            inside = (inp.energy >= energy_range[0]) & (inp.energy <= energy_range[1])
            group = torch.where(inside, group, torch.full_like(group, -1))
        sel = torch.nonzero(group >= 0).flatten()
        # facet ids -> indices into this model's facet table
        ids = np.array(sorted(self.facet_index))
        lut = torch.full((int(ids.max()) + 1,), -1, dtype=torch.int32, device=dev)
        lut[torch.from_numpy(ids).to(dev).long()] = torch.tensor(
            [self.facet_index[int(i)] for i in ids], dtype=torch.int32, device=dev)
        fid = facet_id[sel].long()
        return FrozenPhotons(
            self, pos=inp.pos[:, sel], dir=inp.dir[:, sel], energy=inp.energy[sel],
            weight=out.prob[sel], alpha=alpha[sel], beta=beta[sel], facet=lut[fid],
            order=order[sel].to(torch.int32), group=group[sel].to(torch.int32),
            n_groups=len(orders), theta=theta, rows=sel, process_group=process_group,
            precision=adjoint_precision)


_ADJ_PRECISIONS = {'fp64': 0, 'fp32local': 1}


class FrozenPhotons:
    """Device arrays of the frozen photons and the C-ABI problem over them.

    ``precision``: 'fp64', or 'fp32local' for the moments and gradients of
    a flat-detector chain (float-float positions re-centred on every
    element, float32 reverse sweep, float64 sums; csrc/adjoint32.cu).  The
    freeze (the photons' discrete choices) and ``finite_differences`` run
    in float64 either way.
    """

    def __init__(self, model, pos, dir, energy, weight, alpha, beta, facet, order, group,
                 n_groups, theta=None, stream=None, rows=None, process_group=None,
                 precision='fp64'):
        if n_groups < 1 or n_groups > _abi.ADJ_MAX_GROUPS:
            raise ValueError('pose adjoint: 1..%d groups' % _abi.ADJ_MAX_GROUPS)
        if precision not in _ADJ_PRECISIONS:
            raise ValueError('precision must be one of %s' % list(_ADJ_PRECISIONS))
        if precision == 'fp32local' and model.det_kind != _abi.ADJ_DET_FLAT:
            raise NotImplementedError('FP32-local pose adjoint: flat detectors only '
                                      '(use precision="fp64" for a CircularDetector)')
        self.precision = precision
        self.model = model
        self.rows = rows            # indices of the frozen photons in the traced table
        # photons sharded over the ranks of this torch.distributed group: the
        # moments and the gradient are summed over it (None: one process)
        self.process_group = process_group
        dev = pos.device
        self.device = dev
        f64 = dict(dtype=torch.float64, device=dev)
        self.n = int(pos.shape[1])
        self.n_groups = int(n_groups)
        self.pos = pos.contiguous().to(torch.float64)
        self.dir = dir.contiguous().to(torch.float64)
        self.energy = energy.contiguous().to(torch.float64)
        self.weight = weight.contiguous().to(torch.float64)
        self.alpha = alpha.contiguous().to(torch.float64)
        self.beta = beta.contiguous().to(torch.float64)
        self.facet = facet.contiguous().to(torch.int32)
        self.order = order.contiguous().to(torch.int32)
        self.group = group.contiguous().to(torch.int32)
        self.sign = torch.zeros(self.n, dtype=torch.int8, device=dev)
        self.nsign = torch.zeros(self.n, dtype=torch.int8, device=dev)
        self.root = torch.zeros(self.n, dtype=torch.int8, device=dev)
        self.facets = torch.from_numpy(model.facet_base).to(**f64).contiguous()
        self.flags = torch.from_numpy(model.facet_flags).to(dev).contiguous()
        self.ref = torch.zeros((self.n_groups, 2), **f64)
        # float64 rotations (36 per pose) or FP32-local posed records (24 per element)
        self.rot = torch.empty(max(36 * (model.n_facets + 1), 24 * (model.n_facets + 3)), **f64)
        self.status = torch.zeros(1, dtype=torch.int32, device=dev)
        self.stream = stream
        self._P = None
        self.theta_frozen = model.theta0(dev) if theta is None else \
            torch.as_tensor(theta, dtype=torch.float64, device=dev)
        self._run(self.theta_frozen, _abi.ADJ_FREEZE)
        self.check()
        # moments are taken about the group centres at the frozen parameters
        # (over all shards)
        m = sum_over_shards(self.moments(self.theta_frozen), process_group)
        self.ref = group_centres(m)
        self._P = None

    # ------------------------------------------------------------- launches
    def _problem(self, x_out=None, y_out=None, precision=None):
        P = _abi.MgpuAdjointProblem()
        P.n = self.n
        P.n_facets = self.model.n_facets
        P.n_groups = self.n_groups
        P.det_kind = self.model.det_kind
        P.precision = _ADJ_PRECISIONS[precision or self.precision]
        P.pos, P.dir = self.pos.data_ptr(), self.dir.data_ptr()
        P.alpha, P.beta = self.alpha.data_ptr(), self.beta.data_ptr()
        P.energy, P.weight = self.energy.data_ptr(), self.weight.data_ptr()
        P.facet, P.order, P.group = self.facet.data_ptr(), self.order.data_ptr(), \
            self.group.data_ptr()
        P.sign, P.nsign, P.root = self.sign.data_ptr(), self.nsign.data_ptr(), \
            self.root.data_ptr()
        for name, block in (('lens', self.model.lens_block), ('scatter', self.model.scatter_block),
                            ('det', self.model.det_block)):
            arr = getattr(P, name)
            for k, v in enumerate(block):
                arr[k] = float(v)
        P.facets, P.facet_flags = self.facets.data_ptr(), self.flags.data_ptr()
        P.ref = self.ref.data_ptr()
        P.x_out = x_out.data_ptr() if x_out is not None else None
        P.y_out = y_out.data_ptr() if y_out is not None else None
        P.rot = self.rot.data_ptr()
        P.status = self.status.data_ptr()
        return P

    def _run(self, theta, mode, seeds=None, moments=None, grad=None, x_out=None, y_out=None,
             precision=None):
        theta = self._theta(theta)
        if x_out is None and y_out is None and precision in (None, self.precision):
            if self._P is None or self._P.precision != _ADJ_PRECISIONS[self.precision]:
                self._P = self._problem()
            P = self._P
        else:
            P = self._problem(x_out, y_out, precision)
        lib = _abi.load()
        _abi.check(lib.mgpu_pose_adjoint(C.byref(P), _ptr(theta), mode, _ptr(seeds),
                                         _ptr(moments), _ptr(grad), _stream_handle(self.stream)),
                   'mgpu_pose_adjoint')

    def _theta(self, theta):
        t = torch.as_tensor(theta, dtype=torch.float64, device=self.device)
        if t.shape != (self.model.n_params,):
            raise ValueError('theta must have %d entries' % self.model.n_params)
        return t.contiguous()

    def check(self):
        """Raise if a launch flagged a bad index or a photon without a cylinder root."""
        st = int(self.status.item())
        if st & _abi.STATUS_ADJ_RANGE:
            self.status.zero_()
            raise ValueError('pose adjoint: facet or group index out of range, or a photon '
                             'that meets the detector cylinder at no root')

    def moments(self, theta, out=None):
        """(G, 5) moments: sum w, sum w x', sum w y', sum w x'^2, sum w y'^2
        with (x', y') = detector coordinates minus the group centre ``ref``."""
        m = torch.zeros((self.n_groups, _abi.ADJ_NMOM), dtype=torch.float64,
                        device=self.device) if out is None else out
        self._run(theta, _abi.ADJ_FORWARD, moments=m)
        return m

    def xy(self, theta):
        x = torch.empty(self.n, dtype=torch.float64, device=self.device)
        y = torch.empty_like(x)
        m = torch.zeros((self.n_groups, _abi.ADJ_NMOM), dtype=torch.float64, device=self.device)
        self._run(theta, _abi.ADJ_FORWARD, moments=m, x_out=x, y_out=y)
        return x, y

    def vjp(self, theta, grad_moments):
        """dL/dtheta from dL/dmoments (G, 5)."""
        g = grad_moments.to(torch.float64)
        seeds = torch.stack([g[:, 1], g[:, 3], g[:, 2], g[:, 4]], 1).contiguous()
        grad = torch.zeros(self.model.n_params, dtype=torch.float64, device=self.device)
        self._run(theta, _abi.ADJ_BACKWARD, seeds=seeds, grad=grad)
        return grad

    # ------------------------------------------------------------ gradients
    def loss_and_grad(self, theta, loss_fn):
        """loss_fn(stats) -> scalar, stats from ``moment_stats``."""
        th = self._theta(theta).detach().requires_grad_(True)
        L = loss_fn(moment_stats(PoseMoments.apply(th, self), self.ref))
        (g,) = torch.autograd.grad(L, th)
        return L.detach(), g

    def finite_differences(self, theta, loss_fn, params=None, h=None):
        """Central differences of loss_fn(stats) on the float64 frozen forward.

        Every evaluation is one forward launch over all frozen photons at
        theta +- h_k e_k; the moments of all evaluations stay on the device
        and the losses are formed in one batched step at the end.
        """
        th = self._theta(theta)
        params = np.arange(self.model.n_params) if params is None else np.asarray(params)
        h = self.model.step_sizes() if h is None else np.asarray(h)
        P = len(params)
        thetas = th.repeat(2 * P, 1)
        hk = torch.from_numpy(h[params]).to(self.device)
        rows = torch.arange(P, device=self.device)
        cols = torch.from_numpy(params).to(self.device)
        thetas[rows, cols] += hk
        thetas[P + rows, cols] -= hk
        mom = torch.zeros((2 * P, self.n_groups, _abi.ADJ_NMOM), dtype=torch.float64,
                          device=self.device)
        for k in range(2 * P):
            self._run(thetas[k], _abi.ADJ_FORWARD, moments=mom[k], precision='fp64')
        L = loss_fn(moment_stats(mom, self.ref))
        return (L[:P] - L[P:]) / (2 * hk)

    # ------------------------------------------------------------- checking
    def torch_dict(self):
        """Host float64 tensors of the frozen problem (keys of the float64
        torch-autograd restatement used to check the kernel)."""
        m = self.model
        cpu = lambda t: t.detach().cpu()
        d = {'P0': cpu(self.pos.T), 'd0': cpu(self.dir.T),
             'lens_c': torch.from_numpy(m.lens_block[0:3]), 'lens_n': torch.from_numpy(m.lens_block[3:6]),
             'lens_ez': torch.from_numpy(m.lens_block[6:9]), 'lens_doff': float(m.lens_block[9]),
             'scat_c': torch.from_numpy(m.scatter_block[0:3]),
             'scat_n': torch.from_numpy(m.scatter_block[3:6]),
             'alpha': cpu(self.alpha), 'beta': cpu(self.beta), 'facet': cpu(self.facet).long(),
             'facet_c': torch.from_numpy(m.facet_base[:, 0:3]),
             'facet_n': torch.from_numpy(m.facet_base[:, 3:6]),
             'facet_l': torch.from_numpy(m.facet_base[:, 6:9]),
             'facet_dneg': torch.from_numpy(m.facet_base[:, 9:12]),
             'facet_d': torch.from_numpy(m.facet_base[:, 12]),
             'sign': cpu(self.sign).double(), 'nsign': cpu(self.nsign).double(),
             'order': cpu(self.order).double(), 'energy': cpu(self.energy),
             'w': cpu(self.weight), 'group': cpu(self.group).long(), 'ref': cpu(self.ref)}
        det = m.det_block
        if m.det_kind == _abi.ADJ_DET_FLAT:
            d.update(det_kind='flat', det_c=torch.from_numpy(det[0:3]),
                     det_n=torch.from_numpy(det[3:6]), det_ey=torch.from_numpy(det[6:9]),
                     det_ez=torch.from_numpy(det[9:12]))
        else:
            d.update(det_kind='cyl', det_c=torch.from_numpy(det[0:3]),
                     det_Minv=torch.from_numpy(det[12:21].reshape(3, 3).copy()),
                     det_R=float(det[21]), det_zoomz=float(det[22]),
                     root=cpu(self.root).double())
        return d


def sum_over_shards(t, process_group=None):
    """In-place sum of ``t`` over the ranks of ``process_group`` (one
    all-reduce; the identity for None)."""
    if process_group is not None:
        import torch.distributed as dist
        dist.all_reduce(t, op=dist.ReduceOp.SUM, group=process_group)
    return t


def group_centres(m):
    """(G, 2) weighted centroids from (G, 5) moments taken about the origin."""
    W = m[:, 0].clamp_min(1e-300)
    return torch.stack([m[:, 1] / W, m[:, 2] / W], 1).contiguous()


class PoseMoments(torch.autograd.Function):
    """theta -> (G, 5) detector moments of frozen photons; the backward is
    one launch of the hand-written adjoint.

    Data-parallel over photon shards (``frozen.process_group``): moments are
    sums over photons, so the forward sums them over the ranks; the loss
    and its seeds dL/dmoments are then the same on every rank, each rank's
    backward runs the adjoint on its own photons, and the gradient is
    summed over the ranks -- one all-reduce of G x 5 values and one of the
    parameter vector per gradient."""

    @staticmethod
    def forward(ctx, theta, frozen):
        ctx.frozen = frozen
        ctx.save_for_backward(theta)
        return sum_over_shards(frozen.moments(theta.detach()),
                               getattr(frozen, 'process_group', None))

    @staticmethod
    def backward(ctx, grad_moments):
        (theta,) = ctx.saved_tensors
        g = ctx.frozen.vjp(theta.detach(), grad_moments)
        return sum_over_shards(g, getattr(ctx.frozen, 'process_group', None)), None


def moment_stats(m, ref):
    """W, centroid x, centroid y, variance x, variance y per group (batched
    over leading dims of ``m``)."""
    W = m[..., 0]
    ex = m[..., 1] / W
    ey = m[..., 2] / W
    return {'W': W, 'mean_x': ref[:, 0] + ex, 'mean_y': ref[:, 1] + ey,
            'var_x': m[..., 3] / W - ex * ex, 'var_y': m[..., 4] / W - ey * ey}


def spot_loss(x_nominal, group=0):
    """RMS cross-dispersion width of one group's spot + squared offset of its
    dispersion centroid from ``x_nominal`` (mm)."""
    def loss(s):
        return torch.sqrt(s['var_y'][..., group]) + (s['mean_x'][..., group] - x_nominal) ** 2
    return loss


def resolving_power(zero_group, groups):
    """Mean resolving power x-centroid distance / FWHM over ``groups``, the
    distance taken from the centroid of ``zero_group`` (order 0)."""
    groups = list(groups)

    def rp(s):
        d = (s['mean_x'][..., groups] - s['mean_x'][..., zero_group:zero_group + 1]).abs()
        return (d / (FWHM_PER_SIGMA * torch.sqrt(s['var_x'][..., groups]))).mean(-1)
    return rp


def design_loop(model, photons, orders, zero_order=0, steps=50, lr=0.2, rot_scale=1e-4,
                trans_scale=0.5, optimise=('facet_rotation', 'detector_translation',
                                           'detector_rotation'),
                precision='fp32local', seed=0, min_photons=20, theta_init=None, callback=None,
                process_group=None, row_base=0):
    """Adam on the poses of the chain, maximising the mean resolving power of
    ``orders`` (distance from the ``zero_order`` centroid over FWHM).

    With ``process_group`` every rank holds a shard of the photons (global
    ids from ``row_base``): moments, gradients and the per-order photon
    counts are summed over the ranks, so all ranks take the same steps.

    Every step re-poses the elements at the current parameters, traces
    ``photons`` (host columns or DevicePhotons) with fresh Philox draws, freezes
    the trace and takes the gradient through the adjoint.  Parameters are
    optimised in units of ``rot_scale`` (rad) and ``trans_scale`` (mm),
    starting from ``theta_init`` (default: nominal).  The elements are left
    at the nominal poses on return; the result holds the final theta and
    per-step history.
    """
    import time
    dev = photons.pos.device if hasattr(photons, 'pos') else torch.device('cuda')
    theta0 = model.theta0(dev)
    sl = model.param_slices()
    idx = torch.from_numpy(np.concatenate([sl[k] for k in optimise])).to(dev)
    scale = torch.full((len(idx),), trans_scale, dtype=torch.float64, device=dev)
    rot_keys = {'facet_rotation', 'detector_rotation'}
    off = 0
    for k in optimise:
        if k in rot_keys:
            scale[off:off + len(sl[k])] = rot_scale
        off += len(sl[k])
    base = theta0.clone()
    if theta_init is not None:
        base = torch.as_tensor(theta_init, dtype=torch.float64, device=dev).clone()
    u = ((base - theta0)[idx] / scale).clone().requires_grad_(True)
    base[idx] = theta0[idx]
    opt = torch.optim.Adam([u], lr=lr)
    all_orders = list(orders) + [zero_order]
    history = []
    try:
        for step in range(steps):
            t0 = time.perf_counter()
            theta = base.clone()
            theta[idx] += scale * u.detach()
            model.apply(theta)
            fr, _ = model.trace(photons, all_orders, precision=precision, rng='philox',
                                seed=seed + step, theta=theta, device=dev,
                                process_group=process_group, row_base=row_base)
            counts = sum_over_shards(torch.bincount(fr.group.long(), minlength=len(all_orders)),
                                     process_group).cpu().numpy()
            groups = [g for g in range(len(orders)) if counts[g] >= min_photons]
            rp = resolving_power(len(orders), groups)
            th = theta.detach().requires_grad_(True)
            R = rp(moment_stats(PoseMoments.apply(th, fr), fr.ref))
            (gt,) = torch.autograd.grad(-R, th)
            opt.zero_grad()
            u.grad = gt[idx] * scale
            opt.step()
            torch.cuda.synchronize(dev)
            rec = {'step': step, 'resolving_power': float(R.detach()), 'photons_in_loss': fr.n,
                   'seconds': time.perf_counter() - t0,
                   'peak_bytes': torch.cuda.max_memory_allocated(dev)}
            history.append(rec)
            if callback is not None:
                callback(rec)
            del fr
    finally:
        model.restore()
    theta = base.clone()
    theta[idx] += scale * u.detach()
    return {'theta': theta, 'history': history}


class GraphedGradient:
    """loss_fn(stats) and dL/dtheta of frozen photons as one CUDA graph.

    The forward launch, the torch loss over the moments, the autograd step
    and the reverse launch are captured once; each call copies theta into
    the captured input and replays the graph, so a gradient costs the two
    kernels and no host-side dispatch.  The frozen photons, their group
    centres and ``loss_fn`` are fixed at capture time.
    """

    def __init__(self, frozen, loss_fn, theta=None, warmup=3):
        if getattr(frozen, 'process_group', None) is not None:
            raise ValueError('GraphedGradient captures one process; call loss_and_grad for '
                             'photons sharded over a process group')
        self.frozen = frozen
        dev = frozen.device
        self.theta = (frozen.model.theta0(dev) if theta is None else
                      torch.as_tensor(theta, dtype=torch.float64, device=dev)).clone()
        side = torch.cuda.Stream(device=dev)
        side.wait_stream(torch.cuda.current_stream(dev))
        old = frozen.stream
        frozen.stream = side
        try:
            with torch.cuda.stream(side):
                for _ in range(warmup):
                    frozen.loss_and_grad(self.theta, loss_fn)
            torch.cuda.current_stream(dev).wait_stream(side)
            self.graph = torch.cuda.CUDAGraph()
            with torch.cuda.graph(self.graph, stream=side):
                self.loss, self.grad = frozen.loss_and_grad(self.theta, loss_fn)
        finally:
            frozen.stream = old

    def __call__(self, theta):
        self.theta.copy_(torch.as_tensor(theta, dtype=torch.float64, device=self.theta.device))
        self.graph.replay()
        return self.loss, self.grad
