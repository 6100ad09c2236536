"""PhotonTable, the astropy Table stand-in of the table path (no GPU)."""
import numpy as np

from marxs_gb300 import PhotonTable


def _cols(n=5):
    return {'pos': np.tile([0., 0, 0, 1], (n, 1)), 'dir': np.tile([-1., 0, 0, 0], (n, 1)),
            'energy': np.linspace(0.3, 2, n), 'probability': np.ones(n)}


def test_columns_are_copied_in_order():
    d = _cols()
    t = PhotonTable(d)
    assert t.colnames == ['pos', 'dir', 'energy', 'probability'] and len(t) == 5
    d['energy'][0] = 99.0
    assert t['energy'][0] != 99.0
    t['order'] = 3
    assert t.colnames[-1] == 'order' and np.array_equal(t['order'], np.full(5, 3))
    t.remove_column('order')
    assert 'order' not in t


def test_row_selection_and_copy_are_independent():
    t = PhotonTable(_cols(), meta={'EXPOSURE': 10.0})
    sub = t[np.array([True, False, True, False, True])]
    assert len(sub) == 3 and sub.meta == t.meta and sub.colnames == t.colnames
    c = t.copy()
    c['energy'][:] = 0
    c.meta['EXPOSURE'] = 1.0
    assert np.all(t['energy'] > 0) and t.meta['EXPOSURE'] == 10.0


def test_built_from_another_table_like_object():
    t = PhotonTable(_cols())
    u = PhotonTable(t)
    assert u.colnames == t.colnames
    for k in t.colnames:
        assert np.array_equal(u[k], t[k]) and u[k] is not t[k]
