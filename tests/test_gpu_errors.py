"""Failure paths and column semantics of the GPU backend.

Errors are injected on the host (bad tables, bad inputs, missing draws);
nothing here faults the GPU.  The kernels report through the status word,
which the host maps to the reference's exceptions:
* probability factor outside [0, 1] -> ValueError (optics/base.py:43-46);
* non-homogeneous inputs -> ValueError (geometry.py:495-496 for directions).
Column semantics follow add_output_cols (base/base.py:249-286): a stage
with no hit adds no columns; existing columns keep their values for photons
a stage misses.
"""
import io

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _table(d):
    from marxs_gb300 import PhotonTable
    return PhotonTable({k: np.array(v, copy=True) for k, v in d.items()})


def _photons(n=16):
    from kat_cases import test_photons
    ph = test_photons(n)
    ph['pos'][:, 1] = np.linspace(-1, 1, n)
    return ph


def test_probability_above_one_raises_value_error():
    from marxs_gb300 import FlatGrating, EfficiencyFile
    from marxs_gb300.gpu import GpuSequence
    table = np.array([[0.5, 0.6, 0.9], [2.0, 0.1, 0.2]])          # first row sums to 1.5
    g = FlatGrating(d=1e-3, order_selector=EfficiencyFile(table, [0, 1]), zoom=5)
    ph = _photons()
    for precision in ('fp64', 'fp32local'):
        with pytest.raises(ValueError, match='probability'):
            GpuSequence([g], precision=precision, rng='philox')(_table(ph))


def test_non_homogeneous_direction_raises_value_error():
    from marxs_gb300 import FlatDetector
    from marxs_gb300.gpu import GpuSequence
    ph = _photons()
    ph['dir'][3, 3] = 1.0
    with pytest.raises(ValueError, match='direction'):
        GpuSequence([FlatDetector(zoom=5)])(_table(ph))


def test_missing_predrawn_draws_raise():
    from marxs_gb300 import FlatGrating, OrderSelector
    from marxs_gb300.gpu import GpuSequence
    g = FlatGrating(d=1e-3, order_selector=OrderSelector([0, 1]), zoom=5)
    with pytest.raises(ValueError, match='draws'):
        GpuSequence([g], rng='predrawn')(_table(_photons()))


def test_unsupported_element_raises_not_implemented():
    """An element class the backend does not implement is refused before
    anything runs (there is no CPU fallback); so is a position-dependent
    grating without local coordinate columns to evaluate its callable on."""
    from marxs_gb300 import FlatGrating, OrderSelector
    from marxs_gb300.optics import FlatOpticalElement
    from marxs_gb300.gpu import GpuSequence

    class Baffle(FlatOpticalElement):
        pass
    with pytest.raises(NotImplementedError):
        GpuSequence([Baffle(zoom=5)], rng='philox')(_table(_photons()))
    g = FlatGrating(d=lambda intercoos: np.full(len(intercoos), 1e-3),
                    order_selector=OrderSelector([1]), zoom=5)
    g.loc_coos_name = None
    with pytest.raises(NotImplementedError):
        GpuSequence([g], rng='philox')(_table(_photons()))


def test_stage_without_hits_adds_no_columns():
    from marxs_gb300 import FlatDetector
    from marxs_gb300.gpu import GpuSequence
    det = FlatDetector(zoom=5, position=[0, 100, 0])       # off to the side: no photon hits
    out = GpuSequence([det])(_table(_photons()))
    assert 'det_x' not in out.colnames and 'detpix_x' not in out.colnames
    np.testing.assert_array_equal(np.asarray(out['pos']), _photons()['pos'])


def test_retrace_updates_existing_columns_like_the_reference():
    """Second pass over a table that already has the output columns: only
    photons hit by a stage change, as in the oracle (and MARXS)."""
    from marxs_gb300 import FlatDetector
    from marxs_gb300.gpu import GpuSequence
    from oracle.raytrace import run_sequence
    ph = _photons(40)
    ph['pos'][:, 2] = np.linspace(-4, 4, 40)
    det1 = FlatDetector(zoom=[1, 5, 5], pixsize=0.5)
    det2 = FlatDetector(zoom=[1, 5, 2], pixsize=0.5, position=[-1, 0, 0])   # hits a subset
    ref1, _ = run_sequence([det1], ph)
    ref2, _ = run_sequence([det2], ref1)
    out = GpuSequence([det1])(_table(ph))
    out = GpuSequence([det2])(out)
    assert list(out.colnames) == list(ref2.keys())
    for k in ref2:
        np.testing.assert_allclose(np.asarray(out[k]), ref2[k], rtol=1e-12, atol=1e-12)


def test_chunked_pipeline_equals_single_launch():
    from marxs_gb300 import configs
    from marxs_gb300.gpu import GpuSequence
    inst = configs.build('c2')
    host = configs.photons_for('c2', 50000, seed=4)
    seq = GpuSequence(inst.elements, precision='fp32local', rng='philox', seed=2)
    a = seq(_table(host), chunk=7919)
    b = seq(_table(host), chunk=10 ** 9)
    for k in b.colnames:
        np.testing.assert_array_equal(np.asarray(a[k]), np.asarray(b[k]))
