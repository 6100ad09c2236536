"""Minimal stand-in for the parts of ``astropy`` the MARXS raytrace path uses.

Test infrastructure only (golden-vector generation from the reference in a
container without astropy).  Provides a columnar ``Table`` whose columns are
numpy arrays, a tiny unit system for angles/lengths/energies, and no-op
configuration helpers.
"""
__version__ = '0.0-shim'
