"""GpuSequence with preprocess_steps / postprocess_steps (host logic, no
GPU): like BaseContainer.__call__ (simulator/simulator.py:42-49) the steps
run before and after every element on the photon table.  The one-element
GPU chains are replaced by the oracle here, so the stepwise run must equal
the oracle's run of the whole chain."""
import numpy as np
import pytest

from marxs_gb300 import configs
from marxs_gb300.gpu import GpuSequence


def _sequence(elements, pre, post, seed=3):
    seq = object.__new__(GpuSequence)        # the constructor needs a CUDA device
    seq.elements, seq.preprocess_steps, seq.postprocess_steps = list(elements), pre, post
    seq.precision, seq.rng, seq.seed, seq.device, seq._stepwise = 'fp64', 'predrawn', seed, None, None
    return seq


class _OracleElement:
    """Stands in for a one-element GPU chain: the oracle on the table, in place."""

    def __init__(self, elem, log):
        self.elem, self.log = elem, log

    def __call__(self, table, draws=None, row_base=0, chunk=None):
        from oracle.raytrace import run_sequence
        out, _ = run_sequence([self.elem], table.as_dict(), draws)
        for k, v in out.items():
            table[k] = v
        self.log.append(('elem', type(self.elem).__name__))
        return table


def test_steps_run_around_every_element(monkeypatch):
    from marxs_gb300 import PhotonTable
    from oracle.raytrace import run_sequence
    inst = configs.build('c1')
    n = 2000
    photons = configs.photons_for('c1', n, seed=5)
    draws = configs.draws_for(inst.draw_slots, n, seed=5)
    log = []
    pre = [lambda t: log.append(('pre', len(t.colnames)))]
    post = [lambda t: log.append(('post', len(t.colnames)))]
    seq = _sequence(inst.elements, pre, post)
    made = []
    monkeypatch.setattr(GpuSequence, '_element_sequence',
                        lambda self, k, e: made.append((k, e)) or _OracleElement(e, log))
    out = seq(PhotonTable(photons), draws=draws)
    ref, _ = run_sequence(inst.elements, photons, draws)
    assert [m[1] for m in made] == inst.elements
    kinds = [x[0] for x in log]
    assert kinds == ['pre', 'elem', 'post'] * len(inst.elements)
    # the steps see the table grow: before and after each element
    sizes = [x[1] for x in log if x[0] != 'elem']
    assert sizes == sorted(sizes) and sizes[0] == len(photons) and sizes[-1] == len(ref)
    for col in ('facet', 'order', 'det_x', 'pos'):
        assert np.array_equal(np.asarray(out[col]), ref[col], equal_nan=True), col
    # the one-element chains are made once and reused while the elements stay
    seq(PhotonTable(photons), draws=draws)
    assert len(made) == len(inst.elements)


def test_element_chains_get_distinct_seeds():
    seq = _sequence([], [], [], seed=11)
    seeds = set()
    captured = {}

    def fake_init(self, elements, precision='fp64', rng='predrawn', seed=0, device=None,
                  preprocess_steps=None, postprocess_steps=None):
        captured['seed'] = seed
    orig = GpuSequence.__init__
    try:
        GpuSequence.__init__ = fake_init
        for k in range(4):
            seq._element_sequence(k, object())
            seeds.add(captured['seed'])
    finally:
        GpuSequence.__init__ = orig
    assert len(seeds) == 4 and 11 not in seeds


def test_steps_must_be_callable():
    from marxs_gb300.simulator import SimulationSetupError
    with pytest.raises(SimulationSetupError):
        GpuSequence([], preprocess_steps=[3])
