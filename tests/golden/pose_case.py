"""A Parallel of CAT facets for the pose tests (test infrastructure): the
inputs and a builder that works with the reference's classes and with this
package's."""
import numpy as np


def pose_case():
    """A 6 x 5 array of CAT facets with per-facet rotations and groove
    angles inside a Parallel with its own pose: the inputs to rebuild it."""
    rng = np.random.default_rng(47)
    ys = (np.arange(6) - 2.5) * 27.
    zs = (np.arange(5) - 2.) * 27.
    yy, zz = np.meshgrid(ys, zs, indexing='ij')
    positions = np.stack([np.zeros(yy.size), yy.ravel(), zz.ravel()], axis=1)
    angles = rng.normal(0, 0.02, (yy.size, 3))
    groove = rng.choice([0.0, 0.3, -0.7], yy.size)
    return {'positions': positions, 'angles': angles, 'groove': groove,
            'par_position': np.array([1500., 12., -7.]), 'par_angles': np.array([0.01, -0.02, 0.5]),
            'zoom': np.array([1., 12.5, 12.5]), 'blaze': 0.0314}


def build_pose_parallel(ns, case, euler2mat):
    orient = [euler2mat(*a, 'sxyz') for a in case['angles']]
    grooves = [float(g) for g in case['groove']]
    return ns.Parallel(elem_class=ns.CATGrating,
                       elem_args={'d': 2e-4, 'zoom': list(case['zoom']),
                                  'orientation': euler2mat(0., float(case['blaze']), 0., 'sxyz'),
                                  'order_selector': ns.OrderSelector([-1, 0, 1]),
                                  'groove_angle': grooves},
                       elem_pos={'position': list(case['positions']), 'orientation': orient},
                       position=case['par_position'],
                       orientation=euler2mat(*case['par_angles'], 'sxyz'), id_col='facet')
