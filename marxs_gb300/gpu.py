"""``GpuSequence``: the drop-in GPU backend for a MARXS element chain.

``GpuSequence(elements=[...])(photons)`` behaves like
``marxs.simulator.Sequence(elements=[...])(photons)`` (simulator.py:42-49)
for the supported element classes: the photon table is modified in place
and returned, with the reference's output columns, dtypes and NaN / -1
defaults; a stage that hits no photon adds no columns (optics/base.py:
176-177).  All per-photon arithmetic runs in the CUDA library; PyTorch only
allocates device memory and provides the stream.

Randomness: ``rng='predrawn'`` takes per-photon arrays in ``draws``
(``{element: {'inplanescatter': a, 'perpplanescatter': b}}`` for a
RadialMirrorScatter, ``{element_or_parallel: {'order_u': u}}`` for a grating
stage); ``rng='philox'`` draws in-kernel from Philox4x32-10 keyed by
(seed, photon row, stage index).

``precision='fp64'`` is the parity mode; ``'fp32local'`` runs the ray
arithmetic in float32 in each element's local frame.
"""
import ctypes as C

import numpy as np
import torch

from . import _abi
from .lowering import ChangeWatch, lower_elements, classnames

_PRECISIONS = {'fp64': _abi.FP64, 'fp32local': _abi.FP32LOCAL}
_RNGS = {'predrawn': _abi.RNG_PREDRAWN, 'philox': _abi.RNG_PHILOX}


def _device(device):
    if device is None:
        device = torch.device('cuda', torch.cuda.current_device())
    device = torch.device(device)
    if device.type != 'cuda':
        raise ValueError('GpuSequence runs on a CUDA device only')
    return device


def _stream_handle(stream=None):
    s = torch.cuda.current_stream() if stream is None else stream
    return C.c_void_p(s.cuda_stream)


class DevicePhotons:
    """Device-resident photon state in structure-of-arrays form.

    ``pos``, ``dir``, ``pol`` are ``(3, N)`` float64 planes; ``energy`` and
    ``prob`` are ``(N,)`` float64.
    """

    def __init__(self, n, device=None, empty=False):
        device = _device(device)
        self.n = int(n)
        mk = torch.empty
        self.pos = mk((3, self.n), dtype=torch.float64, device=device)
        self.dir = mk((3, self.n), dtype=torch.float64, device=device)
        self.pol = mk((3, self.n), dtype=torch.float64, device=device)
        self.energy = mk((self.n,), dtype=torch.float64, device=device)
        self.prob = mk((self.n,), dtype=torch.float64, device=device)

    @classmethod
    def from_columns(cls, photons, device=None):
        """From (N,4) homogeneous ``pos``/``dir``/``polarization`` + 1-d columns."""
        n = len(photons['energy'])
        out = cls(n, device)
        for name, key in (('pos', 'pos'), ('dir', 'dir'), ('pol', 'polarization')):
            a = np.asarray(photons[key], dtype=np.float64)[:, :3].T
            getattr(out, name).copy_(torch.from_numpy(np.ascontiguousarray(a)))
        out.energy.copy_(torch.from_numpy(np.ascontiguousarray(photons['energy'], dtype=np.float64)))
        out.prob.copy_(torch.from_numpy(np.ascontiguousarray(photons['probability'],
                                                             dtype=np.float64)))
        return out

    def abi(self):
        return (_abi.vec_soa(self.pos), _abi.vec_soa(self.dir), _abi.vec_soa(self.pol),
                _abi.col(self.energy), _abi.col(self.prob))

    def nbytes(self):
        return 11 * 8 * self.n


class _Instrument:
    """Device copy of the lowered chain: facet tables, selectors, grids."""

    def __init__(self, stages, device, stream):
        from . import lowering as L
        self.stages = stages
        self.device = device
        self.keep = []            # device tensors referenced by raw pointers
        self.stage_facets = {}
        self.stage_selectors = {}
        self.stage_grid = {}
        self.stage_grid_bufs = {}     # si -> (cell_start, cell_items)
        self.stage_aux = {}       # FP32-local constant blocks (bytes, inline in the stage)
        self.stage_sel0 = {}      # first selector of a facet stage (inline copy)
        self.stage_facet_cyl = {} # gratings on Cylinder surfaces: per-facet cylinder blocks
        self.stage_facets32 = {}
        self.stage_table = {}
        self.fp32_error = None
        lib = _abi.load()
        status = torch.zeros(1, dtype=torch.int32, device=device)

        def dev_bytes(raw):
            t = torch.from_numpy(np.frombuffer(raw, dtype=np.uint8).copy()).to(device)
            self.keep.append(t)
            return t

        def spline_struct(sp):
            out = _abi.MgpuSpline1()
            if sp is None:
                return out
            ts = [torch.from_numpy(np.ascontiguousarray(a, dtype=np.float64)).to(device)
                  for a in sp]
            # float copy of the coefficients plus one more surface: their sum
            # over the surfaces (an order selector's total, in one evaluation)
            c = np.asarray(sp[2], dtype=np.float64)
            c32 = torch.from_numpy(np.ascontiguousarray(
                np.concatenate([c, c.sum(axis=0, keepdims=True)]), dtype=np.float32)).to(device)
            tff = [torch.from_numpy(L.split_ff_array(a)).to(device) for a in sp[:2]]
            self.keep += ts + [c32] + tff
            out.nx, out.ny, out.n_surf = len(sp[0]), len(sp[1]), int(sp[2].shape[0])
            out.tx, out.ty, out.c = ts[0].data_ptr(), ts[1].data_ptr(), ts[2].data_ptr()
            out.c32 = c32.data_ptr()
            out.tx_ff, out.ty_ff = tff[0].data_ptr(), tff[1].data_ptr()
            return out

        self.stage_spline = {}
        self.stage_stack = {}

        def f64(a):
            t = torch.from_numpy(np.ascontiguousarray(a, dtype=np.float64)).to(device)
            self.keep.append(t)
            return t.data_ptr()

        for si, st in enumerate(stages):
            if st.spline is not None:
                self.stage_spline[si] = spline_struct(st.spline)
            if st.stack is not None:
                k = st.stack
                l1v32 = torch.from_numpy(np.ascontiguousarray(k['l1_vec'], dtype=np.float32)).to(
                    device)
                self.keep.append(l1v32)
                wd_hi, wd_lo = L.split_ff(1.2398419292004202e-06 / float(k['l1_d']))
                te32, tt32 = [torch.from_numpy(np.ascontiguousarray(k[c], dtype=np.float32)).to(
                    device) for c in ('l1_trans_e', 'l1_trans_t')]
                self.keep += [te32, tt32]
                cs = _abi.MgpuCatStack(k['blaze_center'], k['d_blaze_mm'], k['qf'], k['l1_open'],
                                       k['l1_d'], f64(k['l1_vec']), k['l1_selector'],
                                       len(k['l1_trans_e']), f64(k['l1_trans_e']),
                                       f64(k['l1_trans_t']), k['l2_open'], k['l2_shadow'],
                                       k['l2_total'], k['l2_inner'], l1v32.data_ptr(),
                                       float(wd_hi), float(wd_lo))
                cs.qf32 = float(np.float32(k['qf']))
                cs.l2_open32 = float(np.float32(k['l2_open']))
                cs.l2_absorb32 = float(np.float32(k['l2_shadow'] / k['l2_total']))
                cs.l2_inv_inner32 = float(np.float32(1.0 / k['l2_inner']))
                cs.blaze_center32 = float(np.float32(k['blaze_center']))
                cs.d_blaze32 = float(np.float32(k['d_blaze_mm']))
                cs.l1_open_u53 = L.u53_threshold(k['l1_open'])
                cs.l1_trans_e32, cs.l1_trans_t32 = te32.data_ptr(), tt32.data_ptr()
                self.stage_stack[si] = dev_bytes(bytes(cs))
            try:
                if st.kind in (_abi.STAGE_LENS, _abi.STAGE_SCATTER, _abi.STAGE_FLATDET):
                    self.stage_aux[si] = L.flat32_block(st)
                elif st.kind == _abi.STAGE_CYLDET:
                    blk, table = L.cyl32_block(st)
                    self.stage_aux[si] = blk
                    self.stage_table[si] = dev_bytes(table.tobytes())
                elif st.kind in _abi.FACET_STAGES:
                    if st.facet_cyl is not None:
                        raise NotImplementedError('gratings on Cylinder surfaces run in the '
                                                  'float64 mode only')
                    t32 = L.facets32_table(st.facets, detectors=st.kind == _abi.STAGE_DETARRAY)
                    self.stage_facets32[si] = dev_bytes(t32.tobytes())
                    if st.grid is not None:
                        self.stage_aux[si] = L.grid32_block(st.grid)
                    else:
                        self.stage_aux[si] = bytes(_abi.MgpuGrid32())
            except NotImplementedError as exc:
                self.fp32_error = str(exc)
            if st.kind not in _abi.FACET_STAGES:
                continue
            fac = torch.from_numpy(st.facets.view(np.uint8).copy()).to(device)
            self.keep.append(fac)
            self.stage_facets[si] = fac
            if st.facet_cyl is not None:
                self.stage_facet_cyl[si] = f64(st.facet_cyl)
            sel_structs = (_abi.MgpuSelector * len(st.selectors))()
            for k, s in enumerate(st.selectors):
                e = torch.from_numpy(np.ascontiguousarray(s.energy)).to(device)
                cdf = torch.from_numpy(np.ascontiguousarray(s.cdf)).to(device)
                tot = torch.from_numpy(np.ascontiguousarray(s.total)).to(device)
                ords = torch.from_numpy(np.ascontiguousarray(s.orders, dtype=np.int32)).to(device)
                thr = torch.from_numpy(L.selector_thresholds(s).view(np.int64)).to(device)
                self.keep += [e, cdf, tot, ords, thr]
                gd = L.selector_guide(s) if s.kind == _abi.SEL_CDF else None
                gd_ptr = 0
                if gd is not None:
                    gdt = torch.from_numpy(np.ascontiguousarray(gd)).to(device)
                    self.keep.append(gdt)
                    gd_ptr = gdt.data_ptr()
                sel_structs[k] = _abi.MgpuSelector(s.cdf.shape[0], s.cdf.shape[1],
                                                   1 if s.by_energy else 0,
                                                   1 if L.selector_sorted(s) else 0, e.data_ptr(),
                                                   cdf.data_ptr(), tot.data_ptr(), ords.data_ptr(),
                                                   thr.data_ptr(), s.kind, 0,
                                                   spline_struct(s.spline), gd_ptr)
                rows = L.selector_rows32(s)
                if rows is not None:
                    mid = torch.from_numpy(rows[0]).to(device)
                    self.keep.append(mid)
                    sel_structs[k].e_mid = mid.data_ptr()
                    sel_structs[k].e0_f, sel_structs[k].e_scale_f = rows[1], rows[2]
            if len(st.selectors):
                self.stage_sel0[si] = sel_structs[0]
            raw = np.frombuffer(bytes(sel_structs), dtype=np.uint8).copy()
            sel_dev = torch.from_numpy(raw).to(device)
            self.keep.append(sel_dev)
            self.stage_selectors[si] = sel_dev
            if st.grid is not None:
                self.set_grid(si, st.grid, status, stream)
        if self.stage_grid:
            torch.cuda.current_stream().synchronize()
            code = int(status.item())
            if code & (_abi.STATUS_GRID_RANGE | _abi.STATUS_GRID_FULL):
                raise RuntimeError('facet candidate grid build failed (status 0x%x)' % code)

    def set_grid(self, si, g, status, stream):
        """Allocate and build the candidate grid of grating stage ``si`` from
        the parameters ``g`` (``lowering.grid_params``); the FP32-local
        constants follow.  Returns a rebuild function (the same build on the
        stage's current facet table, e.g. after the facets moved)."""
        from . import lowering as L
        lib = _abi.load()
        dev = self.device
        ncell = g['nu'] * g['nv']
        start = torch.zeros(ncell + 1, dtype=torch.int32, device=dev)
        items = torch.zeros(g['capacity'], dtype=torch.int32, device=dev)
        counts = torch.zeros(ncell + 1 + (ncell + 4095) // 4096, dtype=torch.int32, device=dev)
        self.keep += [start, items, counts]
        grid = _abi.MgpuGrid()
        for key in ('o', 'n', 'a', 'b'):
            getattr(grid, key)[:] = [float(x) for x in g[key]]
        grid.u0, grid.v0, grid.cell = g['u0'], g['v0'], g['cell']
        grid.nu, grid.nv = g['nu'], g['nv']
        grid.slope_max, grid.margin = g['slope_max'], g['margin']
        grid.depth[:] = [float(x) for x in g.get('depth', np.zeros(6))]
        grid.depth_lip = float(g.get('depth_lip', 0.0))
        grid.cell_start, grid.cell_items = start.data_ptr(), items.data_ptr()
        grid.capacity = g['capacity']
        self.stage_grid[si] = grid
        self.stage_grid_bufs[si] = (start, items)
        if si in self.stage_facets32:
            self.stage_aux[si] = L.grid32_block(g)
        fac = self.stage_facets[si]
        n = len(self.stages[si].facets)

        def rebuild(stream_handle):
            _abi.check(lib.mgpu_facet_grid_build(fac.data_ptr(), n, C.byref(grid),
                                                 counts.data_ptr(), status.data_ptr(),
                                                 stream_handle), 'mgpu_facet_grid_build')
        rebuild(stream)
        return rebuild

    def fill_stage(self, si, s):
        st = self.stages[si]
        s.kind = st.kind
        s.id_num = st.id_num
        s.frame[:] = [float(x) for x in st.frame]
        s.cyl[:] = [float(x) for x in st.cyl]
        s.p[:] = [float(x) for x in st.p]
        if st.kind in _abi.FACET_STAGES:
            s.n_facets = len(st.facets)
            s.facets = self.stage_facets[si].data_ptr()
            s.selectors = self.stage_selectors[si].data_ptr()
            s.n_selectors = len(st.selectors)
            s.facet_sel0 = int(len(st.selectors) > 0 and int(np.max(st.facets['selector'])) <= 0)
            if si in self.stage_grid:
                s.grid = self.stage_grid[si]
        if si in self.stage_aux:
            blk = self.stage_aux[si]
            if len(blk) > len(s.aux32):
                raise RuntimeError('FP32-local constant block of %d bytes' % len(blk))
            C.memmove(C.addressof(s.aux32), blk, len(blk))
            s.aux_size = len(blk)
        if si in self.stage_sel0:
            s.sel0 = self.stage_sel0[si]
        if si in self.stage_facet_cyl:
            s.facet_cyl = self.stage_facet_cyl[si]
        if si in self.stage_facets32:
            s.facets32 = self.stage_facets32[si].data_ptr()
        if si in self.stage_table:
            s.table = self.stage_table[si].data_ptr()
        if si in self.stage_spline:
            s.spline = self.stage_spline[si]
        if si in self.stage_stack:
            s.stack = self.stage_stack[si].data_ptr()


class ColumnPlan:
    """Which device buffer each stage writes, and who creates each column.

    Mirrors add_output_cols (marxs/base/base.py:249-286): a float column
    starts as NaN, an id column as -1, unless the table already has it.
    """

    def __init__(self, stages, existing=()):
        self.columns = {}      # name -> 'f8' | 'i4'
        self.first_writer = {} # name -> stage index
        self.order = []        # reference column creation order, per stage
        for si, st in enumerate(stages):
            for name in st.out_names:
                if name is None:
                    continue
                if name not in self.columns:
                    self.columns[name] = 'f8'
                    if name not in existing:
                        self.first_writer[name] = si
            if st.id_col is not None:
                if st.id_col not in self.columns:
                    self.columns[st.id_col] = 'i4'
                    if st.id_col not in existing:
                        self.first_writer[st.id_col] = si
            reads = getattr(st, 'reads', None)
            if reads is not None and reads not in self.columns and reads in existing:
                self.columns[reads] = 'i4'          # read from the table, never written
            self.order.append([c for c in st.new_col_order if c is not None])


class GpuSequence:
    """GPU backend for ``Sequence(elements=[...])`` on supported elements."""

    def __init__(self, elements, precision='fp64', rng='predrawn', seed=0, device=None,
                 preprocess_steps=None, postprocess_steps=None):
        if precision not in _PRECISIONS:
            raise ValueError('precision must be one of %s' % list(_PRECISIONS))
        if rng not in _RNGS:
            raise ValueError('rng must be one of %s' % list(_RNGS))
        self.preprocess_steps = list(preprocess_steps or [])
        self.postprocess_steps = list(postprocess_steps or [])
        for e in list(elements) + self.preprocess_steps + self.postprocess_steps:
            if not callable(e):
                from .simulator import SimulationSetupError
                raise SimulationSetupError('{0} is not callable.'.format(str(e)))
        self.elements = list(elements)
        self._stepwise = None
        self.precision = precision
        self.rng = rng
        self.seed = int(seed)
        self.device = _device(device)
        self._inst = None
        self._watch = None
        self.last_hits = None
        self.last_status = 0
        # False: FP32-local chains run the generic stage loop instead of the
        # kernel specialised for their stage sequence (same results)
        self.specialised = True
        # False: facet stages scan all their facets instead of the candidate
        # grid's lists (same results)
        self.use_grid = True
        # True: FP32-local launches are split every 4096 photons the way
        # launches beyond 2^30 photons are (same results)
        self.split_launches = False

    # ------------------------------------------------------------ lowering
    def lower(self, stream=None):
        """The lowered chain, rebuilt when an element, a pose or a watched
        parameter changed since the last call."""
        if self._inst is None or self._watch.changed(self.elements):
            watch = ChangeWatch(self.elements)
            stages = lower_elements(self.elements)
            self._inst = _Instrument(stages, self.device, _stream_handle(stream))
            self._watch = watch
        return self._inst

    @property
    def stages(self):
        return self.lower().stages

    # ------------------------------------------------------------ launch
    def _chain(self, inst, plan, bufs, draws_dev, n, status, hits, row_base=0):
        if self.precision == 'fp32local' and inst.fp32_error:
            raise NotImplementedError(inst.fp32_error)
        chain = _abi.MgpuChain()
        chain.row_base = int(row_base)
        chain.n_stages = len(inst.stages)
        chain.precision = _PRECISIONS[self.precision]
        chain.rng = _RNGS[self.rng]
        chain.seed = self.seed
        chain.status = status.data_ptr()
        chain.hits = hits.data_ptr()
        chain.flags = ((0 if self.specialised else _abi.FLAG_GENERIC) |
                       (0 if self.use_grid else _abi.FLAG_NO_GRID) |
                       (_abi.FLAG_SPLIT_4K if self.split_launches else 0))
        for si, st in enumerate(inst.stages):
            s = chain.stages[si]
            inst.fill_stage(si, s)
            fw = 0
            for k, name in enumerate(st.out_names):
                if name is None:
                    continue
                s.out[k] = _abi.col(bufs[name])
                if plan.first_writer.get(name) == si:
                    fw |= 1 << k
            if st.id_col is not None:
                idb = bufs[st.id_col]
                s.id_out = idb.data_ptr()
                s.id_stride = 1
                if plan.first_writer.get(st.id_col) == si:
                    fw |= 1 << 16
                if idb.dtype == torch.int64:
                    fw |= 1 << 17
            if st.kind == _abi.STAGE_SUPPORT and st.reads in bufs:
                idb = bufs[st.reads]
                if idb.dtype not in (torch.int32, torch.int64):
                    raise ValueError('catsupportbars needs an integer %r column' % st.reads)
                s.id_out = idb.data_ptr()
                s.id_stride = idb.stride(0)
                if idb.dtype == torch.int64:
                    fw |= 1 << 17
            s.first_writer = fw
            if self.rng == 'predrawn' and st.draw_names:
                d = draws_dev.get(si)
                needed = [k for k, name in enumerate(st.draw_names)
                          if st.kind != _abi.STAGE_SCATTER or st.p[k] != 0.0]
                if d is None or any(d[k] is None for k in needed):
                    raise ValueError('rng="predrawn" needs draws %s for %s' % (
                        [st.draw_names[k] for k in needed], type(st.element).__name__))
                for k, t in enumerate(d):
                    if t is not None:
                        if t.numel() != n:
                            raise ValueError('draw arrays must hold one value per photon')
                        s.draw[k] = t.data_ptr()
                s.draw_stride = 1
        return chain

    def _draws_to_device(self, inst, draws, n):
        out = {}
        if self.rng != 'predrawn':
            return out
        draws = draws or {}
        for si, st in enumerate(inst.stages):
            if not st.draw_names:
                continue
            d = draws.get(st.element)
            if d is None:
                continue
            ts = []
            for name in st.draw_names:
                a = d.get(name)
                if a is None:
                    ts.append(None)
                    continue
                if isinstance(a, torch.Tensor):
                    t = a.to(self.device, dtype=torch.float64).contiguous()
                else:
                    a = np.ascontiguousarray(a, dtype=np.float64)
                    if a.shape != (n,):
                        raise ValueError('draw %r must have shape (%d,)' % (name, n))
                    t = torch.from_numpy(a).to(self.device)
                ts.append(t)
            out[si] = ts
        return out

    def _raise_status(self, code):
        self.last_status = code
        if code & _abi.STATUS_PROB_RANGE:
            raise ValueError('Found probability outside of the 0..1 arange.')
        if code & _abi.STATUS_BAD_W:
            raise ValueError('pos must hold points (w = 1); dir and polarization must be '
                             'direction vectors (w = 0).')
        if code & _abi.STATUS_ORDER_EMPTY:
            raise ValueError('order selection: no order has cumulative probability above the draw')
        if code:
            raise RuntimeError('GPU raytrace reported status 0x%x' % code)

    # ------------------------------------------------------------ device path
    def allocate_columns(self, n, existing=(), id_dtype=torch.int32):
        """Device buffers for every output column of the chain (ids int32 by
        default; int64 matches the reference's column dtype)."""
        inst = self.lower()
        plan = ColumnPlan(inst.stages, existing)
        bufs = {}
        for name, kind in plan.columns.items():
            dt = torch.float64 if kind == 'f8' else id_dtype
            bufs[name] = torch.empty(n, dtype=dt, device=self.device)
        return plan, bufs

    def column_bytes(self):
        """Bytes per photon of every stage column the chain writes (f8 = 8,
        id = 4), and of the draws it reads in pre-drawn mode."""
        inst = self.lower()
        plan = ColumnPlan(inst.stages)
        cols = sum(8 if k == 'f8' else 4 for k in plan.columns.values())
        draws = sum(8 * len(st.draw_names) for st in inst.stages) if self.rng == 'predrawn' else 0
        return cols, draws

    def trace_device(self, inp, out, plan, bufs, draws=None, stream=None, status=None, hits=None,
                     row_base=0, lowered=None):
        """Trace device-resident photons (asynchronous on ``stream``).

        ``inp``/``out`` are DevicePhotons (may be the same object); ``plan``
        and ``bufs`` come from ``allocate_columns``.  Returns the device
        status word and hit counters (read them after synchronising).
        ``lowered``: the result of ``lower()`` earlier in the same call, for
        callers that trace many chunks of one call and check the elements
        once.
        """
        inst = self.lower(stream) if lowered is None else lowered
        n = inp.n
        if status is None:
            status = torch.zeros(1, dtype=torch.int32, device=self.device)
        if hits is None:
            hits = torch.zeros(_abi.MAX_STAGES, dtype=torch.int64, device=self.device)
        draws_dev = draws if isinstance(draws, dict) and all(isinstance(k, int) for k in draws) \
            else self._draws_to_device(inst, draws, n)
        chain = self._chain(inst, plan, bufs, draws_dev, n, status, hits, row_base)
        lib = _abi.load()
        ph = _abi.MgpuPhotons()
        ph.n = n
        ph.pos, ph.dir, ph.pol, ph.energy, ph.prob = inp.abi()
        ph.pos_out, ph.dir_out, ph.pol_out, _, ph.prob_out = out.abi()
        keep = []
        if any(st.host_eval for st in inst.stages):
            keep = self._host_evaluate(inst, chain, ph, bufs, n, stream)
        _abi.check(lib.mgpu_trace(C.byref(chain), C.byref(ph), _stream_handle(stream)),
                   'mgpu_trace')
        if keep:
            # the per-photon columns must outlive the launch
            (stream or torch.cuda.current_stream()).synchronize()
        return status, hits

    def _host_evaluate(self, inst, chain, ph_in, bufs, n, stream):
        """Position-dependent grating constants and blaze modifiers
        (FlatGrating.d with a callable _d and custom blaze_angle_modifier,
        optics/grating.py:209-231): MARXS evaluates these Python callables at
        each photon's local coordinates on the facet it hit.  For every such
        grating stage, the chain up to and including that stage is traced
        once (same draws: Philox streams are keyed by photon and stage, so the
        final trace reproduces these hits), the facets' own callables are
        evaluated on the host at the recorded local coordinates, and the
        results go to the stage as per-photon columns (grating_d, blaze_add)
        of the final trace.  Returns the device columns (keep them alive
        until the final trace has run)."""
        lib = _abi.load()
        keep = []
        tmp = DevicePhotons(n, device=self.device)
        # the locate passes count hits and report status into scratch words:
        # the final trace reports both
        scratch_status = torch.zeros(1, dtype=torch.int32, device=self.device)
        scratch_hits = torch.zeros(_abi.MAX_STAGES, dtype=torch.int64, device=self.device)
        for si, st in enumerate(inst.stages):
            if not st.host_eval:
                continue
            prefix = _abi.MgpuChain.from_buffer_copy(chain)
            prefix.n_stages = si + 1
            prefix.status = scratch_status.data_ptr()
            prefix.hits = scratch_hits.data_ptr()
            # the final trace's input state, the locate pass's own output
            ph = _abi.MgpuPhotons.from_buffer_copy(ph_in)
            ph.pos_out, ph.dir_out, ph.pol_out, _, ph.prob_out = tmp.abi()
            _abi.check(lib.mgpu_trace(C.byref(prefix), C.byref(ph), _stream_handle(stream)),
                       'mgpu_trace')
            (stream or torch.cuda.current_stream()).synchronize()
            y = bufs[st.out_names[0]].cpu().numpy()
            z = bufs[st.out_names[1]].cpu().numpy()
            hit = ~np.isnan(y)
            if st.id_col is not None and len(st.facets) > 1:
                ids = bufs[st.id_col].cpu().numpy()
                index = {int(v): k for k, v in enumerate(st.facets['id_num'])}
                fidx = np.full(n, -1, dtype=np.int64)
                fidx[hit] = [index.get(int(v), -1) for v in ids[hit]]
            else:
                fidx = np.where(hit, 0, -1)
            dcol = np.full(n, np.nan)
            bcol = np.zeros(n)
            for k, g in st.host_eval['d'].items():
                m = fidx == k
                if m.any():
                    dcol[m] = g._d(np.column_stack([y[m], z[m]]))
            for k, g in st.host_eval['blaze'].items():
                m = fidx == k
                if m.any():
                    bcol[m] = g.blaze_angle_modifier(np.column_stack([y[m], z[m]]))
            s = chain.stages[si]
            if st.host_eval['d']:
                t = torch.from_numpy(dcol).to(self.device)
                keep.append(t)
                s.grating_d = _abi.col(t)
            if st.host_eval['blaze']:
                t = torch.from_numpy(bcol).to(self.device)
                keep.append(t)
                s.blaze_add = _abi.col(t)
        return keep

    # ------------------------------------------------------------ table path
    def _element_sequence(self, k, elem):
        """One-element chain for element ``k`` of a sequence with steps; its
        Philox streams get their own seed (a one-element chain numbers its
        stage 0, so a shared seed would repeat the draws of other elements)."""
        seed = (self.seed * 1000003 + 7919 * (k + 1)) & 0xffffffffffffffff
        return GpuSequence([elem], precision=self.precision, rng=self.rng, seed=seed,
                           device=self.device)

    def _call_stepwise(self, photons, draws, row_base, chunk):
        """BaseContainer.__call__ (simulator/simulator.py:42-49) with
        ``preprocess_steps`` / ``postprocess_steps``: the steps see the photon
        table before and after every element, so each element runs as its own
        GPU chain on the table (in place) with the steps on the host between."""
        if isinstance(photons, dict):
            from .table import PhotonTable
            photons = PhotonTable(photons)
        # the one-element chains carry this sequence's settings: rebuild them
        # when an element or any of precision, rng, seed, device changed
        key = (self.precision, self.rng, self.seed, str(self.device))
        if self._stepwise is None or self._stepwise[0] != key or \
                len(self._stepwise[1]) != len(self.elements) or any(
                    sub[0] is not e for sub, e in zip(self._stepwise[1], self.elements)):
            self._stepwise = (key, [(e, self._element_sequence(k, e))
                                    for k, e in enumerate(self.elements)])
        for _, sub in self._stepwise[1]:
            for p in self.preprocess_steps:
                p(photons)
            photons = sub(photons, draws=draws, row_base=row_base, chunk=chunk)
            for p in self.postprocess_steps:
                p(photons)
        return photons

    def __call__(self, photons, draws=None, row_base=0, chunk=8_000_000):
        """Trace a photon table (astropy Table, PhotonTable or dict) in place.

        The photons are processed in chunks alternating over two streams:
        each chunk's host-to-device copy, kernel and device-to-host copy are
        queued on its stream, so transfers in both directions overlap with
        compute.  State columns are copied back into the table's own arrays,
        new columns are attached in the order MARXS creates them.  Host
        arrays in pinned memory (``pinned_photons``) make the copies true DMA.
        On an error (raised after the whole call) the table content is
        unspecified, as in MARXS where earlier elements have already written
        their columns when a later one raises.  With ``preprocess_steps`` or
        ``postprocess_steps`` the elements run one at a time, the steps
        between them (``_call_stepwise``); with ``rng='philox'`` each element
        then draws from its own seed, so the draws (and results) differ from
        the fused chain's for the same seed -- the same distributions, a
        different stream.  Pre-drawn randomness gives identical results.
        """
        if self.preprocess_steps or self.postprocess_steps:
            return self._call_stepwise(photons, draws, row_base, chunk)
        import time as _time
        tm = {}
        t0 = _time.perf_counter()
        if isinstance(photons, dict):
            from .table import PhotonTable
            photons = PhotonTable(photons)
        n = len(photons)
        inst = self.lower()
        tm['lower'] = _time.perf_counter() - t0
        dev = self.device
        colnames = list(photons.colnames)
        host = {}
        for key in ('pos', 'dir', 'polarization'):
            a = np.asarray(photons[key])
            if a.shape != (n, 4):
                raise ValueError('pos, dir and polarization must be (N, 4) homogeneous columns')
            host[key] = np.ascontiguousarray(a, dtype=np.float64)
        for key in ('energy', 'probability'):
            host[key] = np.ascontiguousarray(np.asarray(photons[key]), dtype=np.float64)
        if n == 0:
            return photons
        plan = ColumnPlan(inst.stages, existing=set(colnames))
        main = torch.cuda.current_stream(dev)
        dstate = {k: torch.empty(v.shape, dtype=torch.float64, device=dev) for k, v in host.items()}
        bufs = {}
        for name, kind in plan.columns.items():
            if name in colnames:
                a = np.asarray(photons[name]).astype(np.float64 if kind == 'f8' else np.int64)
                bufs[name] = _h2d(a, dev)
            else:
                dt = torch.float64 if kind == 'f8' else torch.int64
                bufs[name] = torch.empty(n, dtype=dt, device=dev)
        status = torch.zeros(1, dtype=torch.int32, device=dev)
        hits = torch.zeros(_abi.MAX_STAGES, dtype=torch.int64, device=dev)
        draws_dev = self._draws_to_device(inst, draws, n)
        # where results go on the host
        targets, fins = {}, []
        for key in ('pos', 'dir', 'polarization', 'probability'):
            targets[key], fin = _host_target(photons, key, dstate[key])
            fins.append(fin)
        for name in plan.columns:
            if name in colnames:
                targets[name], fin = _host_target(photons, name, bufs[name])
                fins.append(fin)
            else:
                targets[name] = torch.empty(bufs[name].shape, dtype=bufs[name].dtype,
                                            pin_memory=True)
        tm['setup'] = _time.perf_counter() - t0
        lib = _abi.load()
        keep_cols = []            # per-photon columns of host-evaluated gratings
        streams = self._side_streams(dev)
        for st_ in streams:
            st_.wait_stream(main)
        for c, a in enumerate(range(0, n, int(chunk))):
            b = min(n, a + int(chunk))
            side = streams[c % len(streams)]
            with torch.cuda.stream(side):
                for k, v in host.items():
                    dstate[k][a:b].copy_(torch.from_numpy(v[a:b]), non_blocking=True)
                sub_bufs = {name: t[a:b] for name, t in bufs.items()}
                sub_draws = {si: [None if t is None else t[a:b] for t in ts]
                             for si, ts in draws_dev.items()}
                chain = self._chain(inst, plan, sub_bufs, sub_draws, b - a, status, hits,
                                    row_base + a)
                chain.flags |= _abi.FLAG_CHECK_W
                ph = _abi.MgpuPhotons()
                ph.n = b - a
                ph.pos = ph.pos_out = _abi.vec_aos(dstate['pos'][a:b])
                ph.dir = ph.dir_out = _abi.vec_aos(dstate['dir'][a:b])
                ph.pol = ph.pol_out = _abi.vec_aos(dstate['polarization'][a:b])
                ph.energy = _abi.col(dstate['energy'][a:b])
                ph.prob = ph.prob_out = _abi.col(dstate['probability'][a:b])
                if any(st.host_eval for st in inst.stages):
                    keep_cols += self._host_evaluate(inst, chain, ph, sub_bufs, b - a, side)
                _abi.check(lib.mgpu_trace(C.byref(chain), C.byref(ph), _stream_handle(side)),
                           'mgpu_trace')
                for key in ('pos', 'dir', 'polarization', 'probability'):
                    targets[key][a:b].copy_(dstate[key][a:b], non_blocking=True)
                for name in plan.columns:
                    targets[name][a:b].copy_(bufs[name][a:b], non_blocking=True)
        for st_ in streams:
            main.wait_stream(st_)
        tm['issued'] = _time.perf_counter() - t0
        main.synchronize()
        tm['done'] = _time.perf_counter() - t0
        code = int(status.item())
        hit_counts = hits.cpu().numpy()[:len(inst.stages)]
        self.last_hits = hit_counts
        self._raise_status(code)
        for fin in fins:
            if fin is not None:
                fin()
        for si, names in enumerate(plan.order):
            if hit_counts[si] == 0:
                continue
            for name in names:
                if name in colnames:
                    continue
                _attach_column(photons, name, targets[name].numpy())
                colnames.append(name)
        tm['total'] = _time.perf_counter() - t0
        self.last_timing = tm
        return photons

    def _side_streams(self, dev):
        if getattr(self, '_streams', None) is None:
            self._streams = [torch.cuda.Stream(dev), torch.cuda.Stream(dev)]
        return self._streams


def _host_target(photons, name, dev_t):
    """Host tensor that receives a device column: the table's own array when
    its dtype and layout allow, else a pinned staging buffer plus a
    finaliser that writes it back."""
    arr = np.asarray(photons[name])
    want = np.dtype(str(dev_t.dtype).replace('torch.', ''))
    if (arr.shape == tuple(dev_t.shape) and arr.flags.writeable and arr.flags.c_contiguous
            and arr.dtype == want):
        return torch.from_numpy(arr), None
    h = torch.empty(dev_t.shape, dtype=dev_t.dtype, pin_memory=True)

    def fin():
        _write_back(photons, name, h.numpy())
    return h, fin


def _attach_column(photons, name, arr):
    """Add a freshly made column without copying it again."""
    from .table import PhotonTable
    if isinstance(photons, PhotonTable):
        photons.columns[name] = arr
        return
    try:
        photons.add_column(arr, name=name, copy=False)
    except TypeError:
        photons[name] = arr


def pinned_photons(n):
    """A PhotonTable whose state columns live in pinned host memory."""
    from .table import PhotonTable
    t = PhotonTable()
    for key, shape in (('pos', (n, 4)), ('dir', (n, 4)), ('energy', (n,)),
                       ('polarization', (n, 4)), ('probability', (n,))):
        t.columns[key] = torch.empty(shape, dtype=torch.float64, pin_memory=True).numpy()
    return t


def _h2d(a, dev):
    a = np.asarray(a)
    if a.dtype != np.float64 and a.dtype.kind == 'f':
        a = a.astype(np.float64)
    t = torch.from_numpy(np.ascontiguousarray(a))
    return t.to(dev, non_blocking=t.is_pinned())


def _write_back(photons, name, value):
    arr = np.asarray(photons[name])
    if arr.shape == value.shape and arr.flags.writeable and arr.dtype.kind == value.dtype.kind:
        arr[...] = value
    else:
        photons[name] = value.astype(arr.dtype) if arr.shape == value.shape else value


# ---------------------------------------------------------------------------
# Geometry entry points on the GPU (same call shapes as the MARXS methods)
# ---------------------------------------------------------------------------
def _vec_in(a, dev):
    t = torch.from_numpy(np.ascontiguousarray(np.asarray(a, dtype=np.float64))).to(dev)
    if t.dim() == 1:
        t = t[None, :]
    return t


def plane_intersect(geometry, dir, pos, device=None):
    """FinitePlane.intersect (marxs/math/geometry.py:211-261) on the GPU.

    ``geometry`` is anything with ``pos4d``; ``dir``/``pos`` are (N, 4).
    Returns (intersect bool (N,), interpos (N, 4), interpos_local (N, 2)).
    """
    from .lowering import plane_frame
    dev = _device(device)
    lib = _abi.load()
    d, p = _vec_in(dir, dev), _vec_in(pos, dev)
    n = d.shape[0]
    frame = (C.c_double * 14)(*[float(x) for x in plane_frame(geometry.pos4d)])
    hit = torch.empty(n, dtype=torch.uint8, device=dev)
    ip = torch.empty((n, 4), dtype=torch.float64, device=dev)
    ip[:, 3] = p[:, 3]
    loc = torch.empty((2, n), dtype=torch.float64, device=dev)
    _abi.check(lib.mgpu_plane_intersect(frame, n, _abi.vec_aos(p), _abi.vec_aos(d), hit.data_ptr(),
                                        _abi.vec_aos(ip), _abi.col(loc[0]), _abi.col(loc[1]),
                                        _stream_handle()), 'mgpu_plane_intersect')
    return hit.bool().cpu().numpy(), ip.cpu().numpy(), loc.T.contiguous().cpu().numpy()


def cylinder_intersect(geometry, dir, pos, device=None):
    """Cylinder.intersect (marxs/math/geometry.py:470-564) on the GPU."""
    from .lowering import cylinder_block
    dirs = np.asarray(dir, dtype=np.float64)
    if not np.all(dirs[..., 3] == 0):
        raise ValueError('First input must be direction vectors.')
    dev = _device(device)
    lib = _abi.load()
    d, p = _vec_in(dirs, dev), _vec_in(pos, dev)
    n = d.shape[0]
    cyl = (C.c_double * 32)(*[float(x) for x in cylinder_block(geometry)])
    hit = torch.empty(n, dtype=torch.uint8, device=dev)
    ip = torch.empty((n, 4), dtype=torch.float64, device=dev)
    loc = torch.empty((2, n), dtype=torch.float64, device=dev)
    _abi.check(lib.mgpu_cylinder_intersect(cyl, n, _abi.vec_aos(p), _abi.vec_aos(d),
                                           hit.data_ptr(), _abi.vec_aos(ip), _abi.col(loc[0]),
                                           _abi.col(loc[1]), _stream_handle()),
               'mgpu_cylinder_intersect')
    hit_np = hit.bool().cpu().numpy()
    ipn = ip.cpu().numpy()
    ipn[:, 3] = np.where(hit_np, 1.0, np.nan)
    return hit_np, ipn, loc.T.contiguous().cpu().numpy()


def parallel_transport(dir_old, dir_new, pol_old, device=None):
    """parallel_transport (marxs/math/polarization.py:151-170) on the GPU;
    (n, 4) or (n, 3) inputs, returns (n, 4) with w = 0."""
    dev = _device(device)
    lib = _abi.load()

    def as4(a):
        a = np.asarray(a, dtype=np.float64)
        if a.shape[-1] == 3:
            a = np.concatenate([a, np.zeros(a.shape[:-1] + (1,))], axis=-1)
        return _vec_in(a, dev)
    d0, d1, pol = as4(dir_old), as4(dir_new), as4(pol_old)
    out = torch.zeros_like(pol)
    _abi.check(lib.mgpu_parallel_transport(d0.shape[0], _abi.vec_aos(d0), _abi.vec_aos(d1),
                                           _abi.vec_aos(pol), _abi.vec_aos(out), _stream_handle()),
               'mgpu_parallel_transport')
    return out.cpu().numpy()
