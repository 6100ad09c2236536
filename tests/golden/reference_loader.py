"""Import the MARXS reference (Python) from its source tree under test shims.

Test infrastructure only: used to generate golden vectors and to cross-check
the oracle in the CPU test suite.  The reference needs ``astropy`` and
``transforms3d``, which are not installed; the stand-ins in ``refshim/``
provide the subset the raytrace path calls.  Nothing on the GPU path imports
this module.
"""
import os
import sys

# MARXS_REFERENCE_ROOT, else a MARXS checkout named ``reference`` beside
# this repository; the tests that need it skip when neither exists
_REPO = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
REFERENCE_ROOT = os.environ.get('MARXS_REFERENCE_ROOT',
                                os.path.join(os.path.dirname(_REPO), 'reference'))
_SHIM = os.path.join(os.path.dirname(os.path.abspath(__file__)), 'refshim')


def available():
    return os.path.isfile(os.path.join(REFERENCE_ROOT, 'marxs', '__init__.py'))


def load():
    """Return the reference ``marxs`` package (raises if it is not present)."""
    if not available():
        raise ImportError('MARXS reference source tree not found at ' + REFERENCE_ROOT)
    if 'marxs' in sys.modules and getattr(sys.modules['marxs'], '_loaded_from_reference', False):
        return sys.modules['marxs']
    for p in (_SHIM, REFERENCE_ROOT):
        if p not in sys.path:
            sys.path.insert(0, p)
    import marxs
    # The reference reads its version from installed package metadata, which
    # a source tree does not have; base.py needs the attribute at import.
    if not hasattr(marxs, '__version__'):
        marxs.__version__ = '0.0.1'
    marxs._loaded_from_reference = True
    import marxs.optics  # noqa: F401
    import marxs.simulator  # noqa: F401
    import marxs.design  # noqa: F401
    import marxs.math.polarization  # noqa: F401
    return marxs
