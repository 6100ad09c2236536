"""The reference's known-answer tests (tests/kat_cases.py) on the GPU, float64
mode, through the C ABI unit entry points and GpuSequence."""
import numpy as np
import pytest

import kat_cases

pytestmark = pytest.mark.gpu


class GpuRunner:
    def __init__(self, precision='fp64'):
        self.precision = precision

    def plane_intersect(self, geometry, dir, pos):
        from marxs_gb300 import gpu
        return gpu.plane_intersect(geometry, dir, pos)

    def cylinder_intersect(self, geometry, dir, pos):
        from marxs_gb300 import gpu
        return gpu.cylinder_intersect(geometry, dir, pos)

    def transport(self, d1, d2, pol):
        from marxs_gb300 import gpu
        return gpu.parallel_transport(d1, d2, pol)

    def trace(self, elements, photons, draws=None):
        from marxs_gb300 import PhotonTable
        from marxs_gb300.gpu import GpuSequence
        seq = GpuSequence(elements=elements, precision=self.precision, rng='predrawn')
        t = seq(PhotonTable({k: np.array(v, copy=True) for k, v in photons.items()}), draws=draws)
        return {k: np.asarray(t[k]) for k in t.colnames}


@pytest.mark.parametrize('case', kat_cases.CASES, ids=lambda c: c.__name__)
def test_known_answer_gpu(case):
    case(GpuRunner())
