"""astropy.stats stand-in (test-only): sigma_clipped_stats from the oracle's
restatement of astropy's published algorithm."""
import os
import sys

_ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.dirname(os.path.dirname(
    os.path.dirname(os.path.abspath(__file__)))))))
if _ROOT not in sys.path:
    sys.path.insert(0, _ROOT)

from oracle.analysis import sigma_clipped_stats as _scs  # noqa: E402


def sigma_clipped_stats(data, sigma=3.0, maxiters=5, **kwargs):
    if kwargs:
        raise NotImplementedError('sigma_clipped_stats stand-in: %s' % sorted(kwargs))
    return _scs(getattr(data, 'value', data), sigma=sigma, maxiters=maxiters)[:3]
