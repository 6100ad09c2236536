"""Minimal stand-in for the ``transforms3d`` package.

Test infrastructure only: it lets the MARXS reference modules import and run
in a container where ``transforms3d`` is not installed, so that golden
vectors can be generated from the reference itself.  Only the functions the
raytrace path touches are provided, each written from the underlying
mathematics (homogeneous affine composition, Gram-Schmidt decomposition,
Rodrigues rotation, static/rotating Euler sequences).
"""
from . import affines, axangles, euler, utils  # noqa: F401
