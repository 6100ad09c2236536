"""Analysis reductions of photon lists on the GPU.

Same names, arguments and results as the reference's
marxs/analysis/gratings.py for the functions that reduce a photon list per
grating order:

* ``resolvingpower_from_photonlist`` (gratings.py:215-270)
* ``effectivearea_from_photonlist`` (gratings.py:333-363)
* ``average_R_Aeff`` (gratings.py:180-212; host arithmetic on the per-order
  arrays)
* ``CaptureResAeff`` and ``CaptureResAeff_CCDgaps`` (gratings.py:389-560)
* ``sigma_clipped_stats``: astropy.stats.sigma_clipped_stats with the
  defaults the reference calls it with (sigma 3, maxiters 5, median centre,
  population std).

``photons`` is any mapping of columns: the device buffers that
``GpuSequence.trace_device`` / ``simulate_events`` fill (torch CUDA tensors,
read in place, no copy) or host arrays (a PhotonTable, astropy Table or
dict; copied to the device once).  One ``mgpu_order_stats`` call computes
every order's statistics; only the per-order results come back to the host.
"""
import ctypes as C

import numpy as np
import torch

from . import _abi

FWHM_PER_SIGMA = 2.3548


class AnalysisError(Exception):
    pass


def _workspace(device, nbytes):
    """A 256-byte aligned device buffer of at least nbytes, allocated on the
    current stream for this call (the caching allocator reuses it; calls on
    different streams never share one)."""
    buf = torch.empty(int(nbytes) + 256, dtype=torch.uint8, device=device)
    ptr = buf.data_ptr()
    return buf, (ptr + 255) & ~255


def _device():
    return torch.device('cuda', torch.cuda.current_device())


def _as_device(a, device, dtypes=(torch.float64,)):
    """A 1-D device tensor of one of ``dtypes`` (converted to the first if
    needed); device tensors of a supported dtype are used in place.  Masked
    entries of a float column (astropy MaskedColumn, numpy masked array)
    become NaN, which the reductions leave out as the reference's masked
    statistics do."""
    if isinstance(a, torch.Tensor):
        t = a if a.device == device else a.to(device)
    else:
        mask = getattr(a, 'mask', None)
        if mask is not None and np.any(mask) and dtypes[0] == torch.float64:
            a = np.ma.MaskedArray(np.asarray(a, dtype=np.float64), mask=mask).filled(np.nan)
        arr = np.asarray(a)
        if arr.dtype == np.bool_:
            arr = arr.astype(np.uint8)
        t = torch.from_numpy(np.ascontiguousarray(arr)).to(device)
    if t.dim() != 1:
        raise ValueError('photon columns must be one-dimensional')
    if t.dtype not in dtypes:
        t = t.to(dtypes[0])
    return t


def order_stats(value, order=None, orders=(0,), probability=None, aeff_mask=None,
                res_filter=False, sigma=3.0, maxiters=5, stream=None, clip=True):
    """Per-order statistics of ``value`` grouped by ``order``.

    Returns a (len(orders), 8) float64 array with the columns
    ``_abi.STATS_MEAN, STATS_MEDIAN, STATS_STD`` (sigma-clipped, finite values
    of the group), ``STATS_N_CLIP`` (values kept), ``STATS_N_MEMBER``
    (photons in the group passing the filter: finite value and probability
    > 0 with ``res_filter``), ``STATS_AEFF`` (sum of probability over the
    group, restricted to ``aeff_mask``), ``STATS_N_FINITE`` and
    ``STATS_ROUNDS``.  ``order=None`` puts every photon in one group;
    ``clip=False`` computes only the counts and sums (statistics NaN).
    """
    if maxiters < 1:
        raise ValueError('maxiters must be at least 1')
    dev = value.device if isinstance(value, torch.Tensor) and value.is_cuda else _device()
    v = _as_device(value, dev)
    n = v.numel()
    o = None
    if order is not None:
        o = _as_device(order, dev, (torch.float64, torch.int32, torch.int64))
        if o.numel() != n:
            raise ValueError('order and value columns differ in length')
    p = None if probability is None else _as_device(probability, dev)
    if p is not None and p.numel() != n:
        raise ValueError('probability and value columns differ in length')
    m = None
    if aeff_mask is not None:
        m = _as_device(aeff_mask, dev, (torch.uint8,)).contiguous()
        if m.numel() != n:
            raise ValueError('aeff mask and value columns differ in length')
    wanted = [float(x) for x in np.atleast_1d(np.asarray(orders, dtype=np.float64))]
    if order is None:
        wanted = [0.0]
    uniq = list(dict.fromkeys(wanted))
    lib = _abi.load()
    s = torch.cuda.current_stream(dev) if stream is None else stream
    out = {}
    for b in range(0, len(uniq), _abi.STATS_MAX_GROUPS):
        grp = uniq[b:b + _abi.STATS_MAX_GROUPS]
        G = len(grp)
        P = _abi.MgpuStatsProblem()
        P.n = n
        P.value = _abi.MgpuCol(v.data_ptr() if n else None, v.stride(0) if n else 1)
        if o is None:
            P.order_type = _abi.ORDER_NONE
        else:
            P.order = o.data_ptr() if n else None
            P.order_stride = o.stride(0) if n else 1
            P.order_type = {torch.float64: _abi.ORDER_F64, torch.int32: _abi.ORDER_I32,
                            torch.int64: _abi.ORDER_I64}[o.dtype]
        P.n_groups = G
        P.prob = _abi.MgpuCol(p.data_ptr() if (p is not None and n) else None,
                              p.stride(0) if (p is not None and n) else 0)
        P.aeff_mask = m.data_ptr() if (m is not None and n) else None
        P.flags = (_abi.STATS_RES_FILTER if res_filter else 0) | \
            (0 if clip else _abi.STATS_AEFF_ONLY)
        P.maxiters = int(maxiters)
        P.sigma = float(sigma)
        for k, x in enumerate(grp):
            P.orders[k] = x
        nbytes = lib.mgpu_order_stats_workspace(n, G)
        if nbytes < 0:
            raise ValueError('bad order_stats size')
        with torch.cuda.device(dev), torch.cuda.stream(s):
            buf, ptr = _workspace(dev, nbytes)
            res = torch.empty(G * _abi.STATS_NRES, dtype=torch.float64, device=dev)
        P.work, P.work_bytes, P.result = ptr, nbytes, res.data_ptr()
        _abi.check(lib.mgpu_order_stats(C.byref(P), C.c_void_p(s.cuda_stream)),
                   'mgpu_order_stats')
        with torch.cuda.stream(s):
            host = res.cpu().numpy().reshape(G, _abi.STATS_NRES)   # synchronises the stream
        del buf
        for k, x in enumerate(grp):
            out[x] = host[k]
    return np.stack([out[x] for x in wanted])


def sigma_clipped_stats(data, sigma=3.0, maxiters=5):
    """(mean, median, std) of the sigma-clipped finite values of ``data``."""
    r = order_stats(data, None, sigma=sigma, maxiters=maxiters)[0]
    return r[_abi.STATS_MEAN], r[_abi.STATS_MEDIAN], r[_abi.STATS_STD]


def _per_order(r, zeropos, orders):
    """The reference's per-order loop on the device results."""
    if zeropos is None:
        z = r[-1]
        if z[_abi.STATS_N_MEMBER] < 20:
            raise AnalysisError('Too few photons in list to determine position of order 0 '
                                'automatically.')
        zeropos = z[_abi.STATS_MEAN]
        r = r[:-1]
    enough = r[:, _abi.STATS_N_MEMBER] > 20
    pos = np.where(enough, r[:, _abi.STATS_MEAN], np.nan)
    std = np.where(enough, r[:, _abi.STATS_STD], np.nan)
    pos = pos.astype(float).reshape(np.shape(orders))
    std = std.astype(float).reshape(np.shape(orders))
    res = np.abs(pos - zeropos) / (std * FWHM_PER_SIGMA)
    return res, pos, std


def resolvingpower_from_photonlist(photons, orders, col='proj_x', zeropos=None,
                                   ordercol='order'):
    """Resolving power, mean position and clipped std of ``col`` per order
    (NaN for orders with 20 photons or fewer)."""
    orders = np.asanyarray(orders)
    groups = list(np.atleast_1d(orders).astype(float))
    if zeropos is None:
        groups.append(0.0)
    r = order_stats(photons[col], photons[ordercol], groups)
    return _per_order(r, zeropos, orders)


def effectivearea_from_photonlist(photons, orders, n_photons, A_geom=1., ordercol='order'):
    """Sum of probability per order / n_photons * A_geom."""
    orders = np.atleast_1d(np.asanyarray(orders))
    r = order_stats(photons['probability'], photons[ordercol], orders.astype(float),
                    probability=photons['probability'], clip=False)
    return r[:, _abi.STATS_AEFF] / n_photons * A_geom


def average_R_Aeff(r, aeff, axis=None):
    """Aeff summed and R averaged with Aeff as weights (NaN R masked)."""
    aeff_avg = aeff.sum(axis=axis)
    res_avg = np.ma.average(np.ma.masked_invalid(r), weights=aeff, axis=axis)
    return res_avg, aeff_avg


def _length(photons):
    """Rows of a photon table or of a dict of columns."""
    if isinstance(photons, dict):
        for v in photons.values():
            return len(v)
        return 0
    return len(photons)


class CaptureResAeff:
    """Resolving power and effective area per order of a photon list, with
    the reference's constructor and result dict (gratings.py:389-501).

    ``aeff_filter(photons)`` returns None (every photon) or a boolean mask
    column; resolving power uses photons with a finite ``dispersion_coord``
    and probability > 0.  Both reductions run in one device call.
    """

    def __init__(self, A_geom=1, order_col='order', orders=np.arange(-10, 11),
                 dispersion_coord='det_x', zeropos=None):
        self.A_geom = A_geom
        self.order_col = order_col
        self.orders = np.asanyarray(orders)
        self.dispersion_coord = dispersion_coord
        self.zeropos = zeropos

    def aeff_filter(self, photons):
        return None

    def __call__(self, photons, n_photons=None):
        if n_photons is None:
            n_photons = _length(photons)
        groups = list(self.orders.astype(float))
        if self.zeropos is None:
            groups.append(0.0)
        r = order_stats(photons[self.dispersion_coord], photons[self.order_col], groups,
                        probability=photons['probability'],
                        aeff_mask=self.aeff_filter(photons), res_filter=True)
        aeff = r[:len(self.orders), _abi.STATS_AEFF] / n_photons * self.A_geom
        try:
            res = _per_order(r, self.zeropos, self.orders)[0]
        except AnalysisError:
            res = np.nan * np.ones(len(self.orders))
        disporders = self.orders != 0
        avggratres, aeffgrat = average_R_Aeff(res[disporders], aeff[disporders])
        aeff0 = np.sum(aeff[~disporders])
        return {'Aeff0': aeff0, 'Aeffgrat': aeffgrat, 'Aeff': aeff,
                'Rgrat': avggratres, 'R': res}


class CaptureResAeff_CCDgaps(CaptureResAeff):
    """CaptureResAeff whose effective area counts only photons with
    ``photons[aeff_filter_col] >= 0`` (gratings.py:504-560)."""

    def __init__(self, aeff_filter_col='CCD_ID', **kwargs):
        super().__init__(**kwargs)
        self.aeff_filter_col = aeff_filter_col

    def aeff_filter(self, photons):
        c = photons[self.aeff_filter_col]
        if isinstance(c, torch.Tensor):
            return (c >= 0).to(torch.uint8)
        return np.asarray(c) >= 0
