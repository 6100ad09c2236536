"""Host side of device tolerancing: this package's Parallel reproduces the
reference's element poses after wiggle / moveglobal / moveindividual
(golden vectors from design/tolerancing.py), and the per-facet composition
the device kernel evaluates, outer T(t + c) R(a) M, gives the same poses."""
import os
import sys
from types import SimpleNamespace

import numpy as np

from conftest import load_golden

sys.path.insert(0, os.path.join(os.path.dirname(__file__), 'golden'))
from pose_case import build_pose_parallel  # noqa: E402


def _native(g):
    from marxs_gb300 import geomath
    from marxs_gb300.optics import CATGrating, OrderSelector
    from marxs_gb300.simulator import Parallel
    ns = SimpleNamespace(Parallel=Parallel, CATGrating=CATGrating, OrderSelector=OrderSelector)
    case = {k: g[k] for k in ('positions', 'angles', 'groove', 'par_position', 'par_angles',
                              'zoom', 'blaze')}
    return build_pose_parallel(ns, case, geomath.euler2mat)


def _uncert(p):
    from marxs_gb300 import geomath
    return [geomath.compose(q[:3], geomath.euler2mat(q[3], q[4], q[5], 'sxyz'), np.ones(3))
            for q in p]


def _pos4d(gas):
    return np.stack([e.geometry.pos4d for e in gas.elements])


def test_parallel_reproduces_reference_tolerancing():
    from marxs_gb300 import geomath
    g = load_golden('poses')
    gas = _native(g)
    assert np.allclose(_pos4d(gas), g['base_pos4d'], rtol=0, atol=1e-12)
    gas.elem_uncertainty = _uncert(g['wiggle_pert'])
    gas.generate_elements()
    assert np.allclose(_pos4d(gas), g['wiggle_pos4d'], rtol=0, atol=1e-12)
    m = g['global_move']
    gas.uncertainty = geomath.compose(m[:3], geomath.euler2mat(*m[3:], 'sxyz'), np.ones(3))
    gas.generate_elements()
    assert np.allclose(_pos4d(gas), g['global_pos4d'], rtol=0, atol=1e-12)
    gas.elem_uncertainty = _uncert(np.tile(g['indiv_move'], (len(gas.elem_pos), 1)))
    gas.generate_elements()
    assert np.allclose(_pos4d(gas), g['indiv_pos4d'], rtol=0, atol=1e-12)


def test_device_composition_restated_on_the_host():
    """outer T(t + c) R(a) M with (c, M) from local_poses: the arithmetic of
    the pose kernel, in numpy."""
    from marxs_gb300 import geomath
    from marxs_gb300.tolerancing import local_poses
    g = load_golden('poses')
    gas = _native(g)
    loc = local_poses(gas)
    outer0 = np.asarray(gas.pos4d) @ np.asarray(gas.uncertainty)
    m = g['global_move']
    outer1 = np.asarray(gas.pos4d) @ geomath.compose(m[:3], geomath.euler2mat(*m[3:], 'sxyz'),
                                                    np.ones(3))
    for pert, outer, key in ((np.zeros((30, 6)), outer0, 'base_pos4d'),
                             (g['wiggle_pert'], outer0, 'wiggle_pos4d'),
                             (g['wiggle_pert'], outer1, 'global_pos4d'),
                             (np.tile(g['indiv_move'], (30, 1)), outer1, 'indiv_pos4d')):
        for i in range(30):
            R = geomath.euler2mat(*pert[i, 3:], 'sxyz')
            L = outer[:3, :3] @ (R @ loc[i, 3:].reshape(3, 3))
            c = outer[:3, :3] @ (pert[i, :3] + loc[i, :3]) + outer[:3, 3]
            assert np.allclose(L, g[key][i, :3, :3], rtol=0, atol=1e-12), (key, i)
            assert np.allclose(c, g[key][i, :3, 3], rtol=1e-13, atol=1e-12), (key, i)
