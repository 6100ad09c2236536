"""Photon generation: the CPU restatement against the reference's own
RandomArbitraryPdf, polarization_vectors and CircleAperture (golden vectors
recorded by tests/golden/make_golden.py), and the host-side set-up of the
device source."""
import numpy as np

from conftest import load_golden


def _geometry(g):
    from marxs_gb300.optics import Geometry
    return Geometry({'pos4d': g['ap_pos4d']})


def test_restatement_reproduces_reference_bitwise():
    from oracle import source as S
    g = load_golden('source')
    geo = _geometry(g)
    out = S.generate(geo['center'], geo['v_y'], geo['v_z'], geo['e_x'], g['phi'],
                     float(g['r_inner']) / np.linalg.norm(geo['v_y']), [-1, 0, 0],
                     (g['x'], g['bin_width'], g['cdf'], g['sortindex'], True), None, g['draws'])
    for k in ('pos', 'dir', 'energy', 'polarization', 'probability'):
        assert np.array_equal(out[k], g['out_' + k]), k


def test_sampler_tables_equal_the_reference():
    from marxs_gb300.source import RandomArbitraryPdf
    g = load_golden('source')
    p = RandomArbitraryPdf(g['x'], g['pdf_in'])
    assert np.array_equal(p.cdf, g['cdf'])
    assert np.array_equal(p.sortindex, g['sortindex'])
    assert np.array_equal(p.bin_width, g['bin_width'])


def test_device_source_parameters():
    """Polarization basis, probability and normalised inner radius as the
    reference derives them (no GPU needed: only host set-up)."""
    import torch
    from marxs_gb300.source import CircleAperture, DeviceSource, RandomArbitraryPdf
    from oracle import source as S
    g = load_golden('source')
    ap = CircleAperture(pos4d=g['ap_pos4d'], r_inner=300., phi=list(g['phi']))
    src = DeviceSource(ap, energy=RandomArbitraryPdf(g['x'], g['pdf_in']), device='cpu')
    v1, v2 = S.polarization_basis([-1, 0, 0])
    assert np.array_equal(src.v1, v1) and np.array_equal(src.v2, v2)
    assert src.prob == 1.0
    assert src.r_inner_norm == 300. / 500.
    tilted = DeviceSource(ap, direction=[-1, 0.2, 0], device='cpu')
    d = np.array([-1, 0.2, 0]) / np.linalg.norm([-1, 0.2, 0])
    assert np.isclose(tilted.prob, -np.dot(d, [1, 0, 0]))
    # a table spectrum becomes the reference's RandomArbitraryPdf input
    t = DeviceSource(ap, energy={'energy': g['x'], 'fluxdensity': np.r_[9., g['pdf_in'][1:]]},
                     device='cpu')
    assert np.array_equal(t.pdf.cdf, g['cdf'])
    assert torch.device('cpu') == src.device
