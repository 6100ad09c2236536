"""CPU restatement of the photon-list analysis reductions (test
infrastructure: only tests and the measurement harness use it).

* ``sigma_clipped_stats`` restates astropy.stats.sigma_clipped_stats, a
  third-party dependency of the reference (``astropy>=6.0.1``,
  pyproject.toml:23) that is not installed here, from its published
  algorithm with the defaults the reference relies on (sigma 3, maxiters 5,
  cenfunc 'median', stdfunc 'std', std_ddof 0, no grow): drop non-finite
  values; repeat up to ``maxiters`` times: centre = median, width = std of
  the current values, keep ``centre - sigma*std <= x <= centre + sigma*std``,
  stop early when nothing was removed; return mean, median and std of the
  values kept.  Its parity against astropy itself is unpinned (astropy is
  absent); the reference's own tests that exercise it through
  resolvingpower_from_photonlist (analysis/tests/test_grating.py:16-80) pin
  it statistically.
* ``resolvingpower_from_photonlist``  analysis/gratings.py:215-270
* ``effectivearea_from_photonlist``   analysis/gratings.py:333-363
* ``average_R_Aeff``                  analysis/gratings.py:180-212
* ``capture_res_aeff``                CaptureResAeff.__call__ with its
  default filters, analysis/gratings.py:430-501
"""
import numpy as np


class AnalysisError(Exception):
    pass


def sigma_clipped_stats(data, sigma=3.0, maxiters=5):
    """(mean, median, std) of the sigma-clipped finite values; also returns
    the number of values kept and of iterations run."""
    x = np.asarray(data, dtype=np.float64).ravel()
    x = x[np.isfinite(x)]
    it = 0
    if x.size == 0:
        return np.nan, np.nan, np.nan, 0, 0
    while it < maxiters:
        it += 1
        size = x.size
        cen = np.median(x)
        std = np.std(x)
        lo = cen - std * sigma
        hi = cen + std * sigma
        x = x[(x >= lo) & (x <= hi)]
        if size - x.size == 0:
            break
    if x.size == 0:
        return np.nan, np.nan, np.nan, 0, it
    return float(np.mean(x)), float(np.median(x)), float(np.std(x)), int(x.size), it


def resolvingpower_from_photonlist(order, value, orders, zeropos=None):
    """Per-order resolving power, mean position and clipped std: a group with
    20 or fewer photons gives NaN; zeropos from the order-0 photons (at least
    20) when not given."""
    order = np.asarray(order)
    value = np.asarray(value, dtype=np.float64)
    orders = np.asarray(orders)
    if zeropos is None:
        ind = order == 0
        if ind.sum() < 20:
            raise AnalysisError('Too few photons in list to determine position of order 0 '
                                'automatically.')
        zeropos = sigma_clipped_stats(value[ind])[0]
    pos = np.zeros_like(orders, dtype=float)
    std = np.zeros_like(orders, dtype=float)
    for i, o in enumerate(orders):
        ind = order == o
        if ind.sum() > 20:
            meanpos, _, stdpos = sigma_clipped_stats(value[ind])[:3]
        else:
            meanpos, stdpos = np.nan, np.nan
        pos[i] = meanpos
        std[i] = stdpos
    res = np.abs(pos - zeropos) / (std * 2.3548)
    return res, pos, std


def effectivearea_from_photonlist(order, probability, orders, n_photons, A_geom=1.):
    order = np.asarray(order)
    probability = np.asarray(probability, dtype=np.float64)
    aeff = np.zeros(len(orders))
    for i, o in enumerate(orders):
        aeff[i] = probability[order == o].sum()
    return aeff / n_photons * A_geom


def average_R_Aeff(r, aeff, axis=None):
    aeff_avg = aeff.sum(axis=axis)
    res_avg = np.ma.average(np.ma.masked_invalid(r), weights=aeff, axis=axis)
    return res_avg, aeff_avg


def capture_res_aeff(order, value, probability, orders, n_photons=None, A_geom=1, zeropos=None,
                     aeff_mask=None):
    """CaptureResAeff()(photons): aeff over the photons in ``aeff_mask`` (all
    by default); R over finite values with probability > 0."""
    order = np.asarray(order)
    value = np.asarray(value, dtype=np.float64)
    probability = np.asarray(probability, dtype=np.float64)
    orders = np.asarray(orders)
    if n_photons is None:
        n_photons = len(order)
    ind = np.ones(len(order), dtype=bool) if aeff_mask is None else np.asarray(aeff_mask)
    aeff = effectivearea_from_photonlist(order[ind], probability[ind], orders, n_photons, A_geom)
    try:
        ind = np.isfinite(value) & (probability > 0)
        res, pos, std = resolvingpower_from_photonlist(order[ind], value[ind], orders, zeropos)
    except AnalysisError:
        res = np.nan * np.ones(len(orders))
    disporders = orders != 0
    avggratres, aeffgrat = average_R_Aeff(res[disporders], aeff[disporders])
    aeff0 = np.sum(aeff[~disporders])
    return {'Aeff0': aeff0, 'Aeffgrat': aeffgrat, 'Aeff': aeff, 'Rgrat': avggratres, 'R': res}
