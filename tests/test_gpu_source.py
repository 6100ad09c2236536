"""Photon generation on the GPU (point source through a CircleAperture).

* pre-drawn mode against the golden vectors recorded from the reference's own
  RandomArbitraryPdf, polarization_vectors and CircleAperture: energy and
  probability bit-exact (same float64 operations), position and polarization
  to 1e-12 (library sin/cos/sqrt differ in the last bit);
* Philox mode follows the reference distributions (KS p > 1e-3 against the
  restatement fed numpy uniforms): energies, aperture radius and angle,
  polarization angle;
* generated photons trace through the CAT array like host-made ones, and
  the Philox streams are keyed by global photon id.
"""
import numpy as np
import pytest
import torch
from scipy import stats

from conftest import load_golden

pytestmark = pytest.mark.gpu


def _source(g, **kw):
    from marxs_gb300.source import CircleAperture, DeviceSource, RandomArbitraryPdf
    ap = CircleAperture(pos4d=g['ap_pos4d'], r_inner=float(g['r_inner']), phi=list(g['phi']))
    return DeviceSource(ap, energy=RandomArbitraryPdf(g['x'], g['pdf_in']), **kw)


def _host(out):
    return {'pos': out.pos.T.cpu().numpy(), 'dir': out.dir.T.cpu().numpy(),
            'polarization': out.pol.T.cpu().numpy(), 'energy': out.energy.cpu().numpy(),
            'probability': out.prob.cpu().numpy()}


def test_predrawn_generation_matches_reference():
    g = load_golden('source')
    n = int(g['n'])
    out = _host(_source(g).generate(n, draws=torch.from_numpy(g['draws']).cuda()))
    assert np.array_equal(out['energy'], g['out_energy'])
    assert np.array_equal(out['probability'], g['out_probability'])
    assert np.array_equal(out['dir'], g['out_dir'][:, :3])
    for k in ('pos', 'polarization'):
        ref = g['out_' + k][:, :3]
        assert np.max(np.abs(out[k] - ref) / np.maximum(np.abs(ref), 1.0)) < 1e-12, k


def test_philox_generation_follows_reference_distributions():
    from oracle import source as S
    g = load_golden('source')
    n = 200_000
    src = _source(g)
    out = _host(src.generate(n, seed=11))
    ref = S.generate(src.center, src.v_y, src.v_z, src.e_x, src.phi, src.r_inner_norm,
                     src.direction, (g['x'], g['bin_width'], g['cdf'], g['sortindex'], True),
                     None, np.random.default_rng(5).random((5, n)))
    assert stats.ks_2samp(out['energy'], ref['energy']).pvalue > 1e-3
    rel = out['pos'] - src.center
    R = np.linalg.norm(src.v_y)
    r = np.hypot(rel @ (src.v_y / R), rel @ (src.v_z / R)) / R
    phi = np.arctan2(rel @ (src.v_z / R), rel @ (src.v_y / R)) % (2 * np.pi)
    ri2 = src.r_inner_norm ** 2
    assert stats.kstest((r ** 2 - ri2) / (1 - ri2), 'uniform').pvalue > 1e-3
    assert stats.kstest((phi - src.phi[0]) / (src.phi[1] - src.phi[0]), 'uniform').pvalue > 1e-3
    ang = np.arctan2(out['polarization'] @ src.v2, out['polarization'] @ src.v1) % (2 * np.pi)
    assert stats.kstest(ang / (2 * np.pi), 'uniform').pvalue > 1e-3
    assert np.max(np.abs(np.linalg.norm(out['polarization'], axis=1) - 1)) < 1e-12


def test_streams_are_keyed_by_global_photon_id():
    g = load_golden('source')
    src = _source(g)
    whole = src.generate(10_000, seed=3)
    half = src.generate(5_000, seed=3, row_base=5_000)
    for a, b in ((whole.pos[:, 5000:], half.pos), (whole.energy[5000:], half.energy),
                 (whole.pol[:, 5000:], half.pol)):
        assert torch.equal(a, b)


def test_generated_photons_trace_like_host_photons():
    """Device photons go through the CAT array; the same photons copied to the
    host and traced through the table API give the same columns."""
    from marxs_gb300 import configs, PhotonTable
    from marxs_gb300.gpu import GpuSequence
    from marxs_gb300.source import CircleAperture, DeviceSource
    inst = configs.build('c2')
    ap = CircleAperture(position=[12000., 0, 0], zoom=[1, 500, 500], r_inner=300.)
    src = DeviceSource(ap, energy={'energy': np.linspace(0.3, 2.0, 40),
                                   'fluxdensity': np.ones(40)})
    n = 100_000
    dev = src.generate(n, seed=9)
    seq = GpuSequence(inst.elements, precision='fp32local', rng='philox', seed=4)
    plan, bufs = seq.allocate_columns(n)
    from marxs_gb300.gpu import DevicePhotons
    out = DevicePhotons(n)
    status, hits = seq.trace_device(dev, out, plan, bufs)
    torch.cuda.synchronize()
    assert int(status.item()) == 0
    assert (bufs['facet'] >= 0).float().mean().item() > 0.3
    host = _host(dev)
    table = PhotonTable({'pos': np.c_[host['pos'], np.ones(n)], 'dir': np.c_[host['dir'], np.zeros(n)],
                         'polarization': np.c_[host['polarization'], np.zeros(n)],
                         'energy': host['energy'], 'probability': host['probability']})
    ref = seq(table)
    assert torch.equal(torch.from_numpy(np.asarray(ref['facet'])).cuda().to(bufs['facet'].dtype),
                       bufs['facet'])
    d = np.asarray(ref['det_phi'])
    a = bufs['det_phi'].cpu().numpy()
    assert np.array_equal(np.isnan(a), np.isnan(d))
    assert np.array_equal(a[~np.isnan(a)], d[~np.isnan(d)])


def test_simulate_events_does_not_depend_on_chunking():
    """The two-stream chunked pipeline gives the event list of one generate +
    trace_device over all photons, whatever the chunk size (ragged last
    chunk included)."""
    from marxs_gb300 import configs
    from marxs_gb300.gpu import DevicePhotons, GpuSequence
    from marxs_gb300.source import CircleAperture, DeviceSource, simulate_events
    inst = configs.build('c2')
    ap = CircleAperture(position=[12000., 0, 0], zoom=[1, 500, 500], r_inner=300.)
    src = DeviceSource(ap, energy={'energy': np.linspace(0.3, 2.0, 40),
                                   'fluxdensity': np.ones(40)})
    seq = GpuSequence(inst.elements, precision='fp32local', rng='philox', seed=4)
    n = 50_000
    cols = ('det_phi', 'det_y', 'order', 'facet')
    ph = src.generate(n, seed=21, row_base=100)
    plan, bufs = seq.allocate_columns(n)
    status, _ = seq.trace_device(ph, ph, plan, bufs, row_base=100)
    torch.cuda.synchronize()
    assert int(status.item()) == 0
    for chunk in (n, 16_384, 7_001):
        ev = simulate_events(src, seq, n, cols, seed=21, row_base=100, chunk=chunk)
        for c in cols:
            assert ev[c].is_pinned()
            a, b = ev[c].numpy(), bufs[c].cpu().numpy()
            assert np.array_equal(a, b, equal_nan=a.dtype.kind == 'f'), (chunk, c)
    with pytest.raises(ValueError):
        simulate_events(src, seq, 10, ('no_such_column',))


def test_fp32local_generation_follows_the_same_distributions():
    """precision='fp32local' (float32 trigonometry, integer energy bins):
    KS against the float64 generator's samples, uniform aperture radius and
    angle and polarization angle, unit polarization, keyed by photon id."""
    g = load_golden('source')
    n = 400_000
    ref = _host(_source(g).generate(n, seed=11))
    src = _source(g, precision='fp32local')
    out = _host(src.generate(n, seed=12))
    assert stats.ks_2samp(out['energy'], ref['energy']).pvalue > 1e-3
    assert np.isin(np.unique(np.floor(out['energy'] * 1e3)), np.floor(ref['energy'] * 1e3)).mean() > 0.99
    rel = out['pos'] - src.center
    R = np.linalg.norm(src.v_y)
    r = np.hypot(rel @ (src.v_y / R), rel @ (src.v_z / R)) / R
    phi = np.arctan2(rel @ (src.v_z / R), rel @ (src.v_y / R)) % (2 * np.pi)
    ri2 = src.r_inner_norm ** 2
    assert stats.kstest((r ** 2 - ri2) / (1 - ri2), 'uniform').pvalue > 1e-3
    assert stats.kstest((phi - src.phi[0]) / (src.phi[1] - src.phi[0]), 'uniform').pvalue > 1e-3
    assert np.abs(rel @ src.e_x).max() < 1e-9                       # in the aperture plane
    ang = np.arctan2(out['polarization'] @ src.v2, out['polarization'] @ src.v1) % (2 * np.pi)
    assert stats.kstest(ang / (2 * np.pi), 'uniform').pvalue > 1e-3
    assert np.max(np.abs(np.linalg.norm(out['polarization'], axis=1) - 1)) < 1e-6
    assert np.array_equal(out['dir'], ref['dir']) and np.array_equal(out['probability'],
                                                                      ref['probability'])
    whole = src.generate(10_000, seed=3)
    half = src.generate(5_000, seed=3, row_base=5_000)
    assert torch.equal(whole.pos[:, 5000:], half.pos) and torch.equal(whole.energy[5000:],
                                                                      half.energy)
    with pytest.raises(ValueError):
        src.generate(10, draws=torch.zeros((5, 10), dtype=torch.float64, device='cuda'))
