"""The check that decides, on every GpuSequence call, whether the chain must
be lowered again (host logic, no GPU): element moves by assignment
(design/tolerancing.py:133) or in place, order selectors swapped on facets
(analysis/gratings.py:117-124), parameters changed, elements replaced --
and nothing when the same values are assigned again."""
import copy

import numpy as np
import pytest

from marxs_gb300 import configs
from marxs_gb300.lowering import ChangeWatch


@pytest.fixture(params=['c2', 'c6'])
def chain(request):
    return configs.build(request.param).elements


def test_unchanged(chain):
    w = ChangeWatch(chain)
    assert not w.changed(chain)
    assert not w.changed(list(chain))


def test_facet_pose_assigned(chain):
    w = ChangeWatch(chain)
    g = chain[2].elements[17].geometry
    move = np.eye(4)
    move[0, 3] = 1e-3
    g.pos4d = move @ g.pos4d
    assert w.changed(chain)


def test_facet_pose_edited_in_place(chain):
    w = ChangeWatch(chain)
    chain[2].elements[500].geometry.pos4d[1, 3] += 1e-9
    assert w.changed(chain)


def test_same_pose_values_assigned_again(chain):
    w = ChangeWatch(chain)
    g = chain[2].elements[3].geometry
    g.pos4d = np.array(g.pos4d, copy=True)
    assert not w.changed(chain)


def test_order_selector_swapped(chain):
    w = ChangeWatch(chain)
    f = chain[2].elements[0]
    if not hasattr(f, 'order_selector'):
        f = f.elements[0]                            # the membrane of a stacked facet
    f.order_selector = copy.copy(f.order_selector)
    assert w.changed(chain)


def test_lens_parameter(chain):
    w = ChangeWatch(chain)
    lens = chain[0]
    lens.focallength = float(lens.focallength)      # same value, new object
    assert not w.changed(chain)
    lens.focallength = lens.focallength + 1.0
    assert w.changed(chain)


def test_elements_replaced(chain):
    w = ChangeWatch(chain)
    assert w.changed(chain[:3])
    par = chain[2]
    par.elements[5] = copy.copy(par.elements[5])
    assert w.changed(chain)


def test_stack_layer_moved():
    chain = configs.build('c6').elements
    w = ChangeWatch(chain)
    facet = chain[2].elements[10]
    layers = getattr(facet, 'elements', None)
    assert layers, 'CATL1L2Stack facets hold their layers as elements'
    layers[1].geometry.pos4d = layers[1].geometry.pos4d.copy()
    assert not w.changed(chain)                      # identity changed, same values
    layers[1].geometry.pos4d[0, 3] += 1e-6
    assert w.changed(chain)


def test_stack_layer_parameters():
    chain = configs.build('c6').elements
    facet = chain[2].elements[4]
    qf = facet.elements[1]
    w = ChangeWatch(chain)
    qf.factor = qf.factor * 0.99
    assert w.changed(chain)
    w = ChangeWatch(chain)
    facet.elements[2].openfraction = facet.elements[2].openfraction * 0.99
    assert w.changed(chain)


def test_lens_reflectivity_and_detector_pixels():
    chain = configs.build('c5').elements
    w = ChangeWatch(chain)
    chain[0].reflectivity_interpolator = configs.lens_reflectivity(99)
    assert w.changed(chain)
    w = ChangeWatch(chain)
    chain[-1].pixsize = chain[-1].pixsize * 2
    assert w.changed(chain)


def test_order_selector_table_edited_in_place(chain):
    """A selector's probability table edited in place (same object, same
    array) must make the chain lower again."""
    w = ChangeWatch(chain)
    f = chain[2].elements[0]
    if not hasattr(f, 'order_selector'):
        f = f.elements[0]
    sel = f.order_selector
    if hasattr(sel, 'cumprob'):                      # EfficiencyFile
        sel.cumprob[..., 0] *= 0.5
    else:                                            # InterpolateEfficiencyTable
        spl = sel.interpolators[3]
        coeff = spl.tck[2] if hasattr(spl, 'tck') else spl.get_coeffs()
        coeff[0] += 1e-3
    assert w.changed(chain)


def test_reflectivity_coefficients_edited_in_place():
    chain = configs.build('c5').elements
    w = ChangeWatch(chain)
    assert not w.changed(chain)
    spl = chain[0].reflectivity_interpolator
    arrays = [a for a in vars(spl).values() if isinstance(a, np.ndarray)]
    arrays += [a for t in vars(spl).values() if isinstance(t, (list, tuple))
               for a in t if isinstance(a, np.ndarray)]
    assert arrays, 'the interpolator keeps its tables as arrays'
    max(arrays, key=lambda a: a.size).flat[0] += 1e-3
    assert w.changed(chain)
