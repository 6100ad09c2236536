"""GB300-native backend for the MARXS photon-raytrace hot path.

Photons stay resident on the GPU through a chain of flat and cylindrical
optical elements (PerfectLens, RadialMirrorScatter, a Parallel array of
FlatGrating/CATGrating facets with nearest-hit lookup, FlatDetector,
CircularDetector).  Hand-written sm_103a CUDA kernels behind a C ABI do the
per-photon work; PyTorch only provides device memory and streams.

Entry point: ``GpuSequence(elements=[...])(photons)``, a drop-in for
``marxs.simulator.Sequence`` on these element classes.
"""
from .optics import (FinitePlane, Cylinder, OrderSelector, EfficiencyFile, PerfectLens,
                     RadialMirrorScatter, FlatDetector, CircularDetector, FlatGrating,
                     CATGrating, GeometryError)
from .simulator import Sequence, Parallel, SimulationSetupError
from .table import PhotonTable

__version__ = '0.1.0'


def __getattr__(name):
    # the GPU entry points load the CUDA library lazily
    if name in ('GpuSequence', 'DevicePhotons'):
        from . import gpu
        return getattr(gpu, name)
    raise AttributeError(name)
