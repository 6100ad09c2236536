"""Reference-style integration checks on the GPU.

* the interface conformance of every element (optics/tests/test_all_optics.py:
  191-214): probability never increases; polarization stays a unit vector
  perpendicular to the direction -- checked after every prefix of the CAT
  chain, in float64 (1e-12) and FP32-local (1e-6);
* the end-to-end pipeline of marxs/tests/test_analysis.py:30-110, through
  this package's own path (photons generated on the device, traced, reduced
  on the device): the resolving power of order -6 is about twice that of
  order -3 (20 %), order 0 has none, and CaptureResAeff agrees with the
  oracle on host copies of the same columns.
"""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize('precision, tol', [('fp64', 1e-12), ('fp32local', 1e-6)])
def test_element_invariants_after_every_stage(precision, tol):
    from marxs_gb300 import configs
    from marxs_gb300.gpu import DevicePhotons, GpuSequence
    from marxs_gb300.optics import catsupportbars
    inst = configs.build('c2')
    chain = inst.elements[:3] + [catsupportbars] + inst.elements[3:]
    n = 100_000
    host = configs.photons_for('c2', n, seed=17)
    p_in = host['probability']
    for k in range(1, len(chain) + 1):
        seq = GpuSequence(chain[:k], precision=precision, rng='philox', seed=2)
        ph = DevicePhotons.from_columns(host)
        plan, bufs = seq.allocate_columns(n)
        status, _ = seq.trace_device(ph, ph, plan, bufs)
        torch.cuda.synchronize()
        assert int(status.item()) == 0
        prob = ph.prob.cpu().numpy()
        d = ph.dir.T.cpu().numpy()
        q = ph.pol.T.cpu().numpy()
        assert np.all(prob <= p_in) and np.all(prob >= 0), k
        d = d / np.linalg.norm(d, axis=1)[:, None]
        assert np.max(np.abs(np.linalg.norm(q, axis=1) - 1)) < tol, k
        assert np.max(np.abs(np.einsum('ij,ij->i', q, d))) < tol, k


@pytest.mark.parametrize('precision', ['fp64', 'fp32local'])
def test_resolving_power_pipeline(precision):
    from marxs_gb300 import configs
    from marxs_gb300.analysis import CaptureResAeff
    from marxs_gb300.gpu import GpuSequence
    from marxs_gb300.source import CircleAperture, DeviceSource
    from oracle import analysis as A
    inst = configs.build('c2')
    ap = CircleAperture(position=[12000., 0, 0], zoom=[1, 500, 500], r_inner=300.)
    src = DeviceSource(ap, energy=0.5)
    seq = GpuSequence(inst.elements, precision=precision, rng='philox', seed=8)
    n = 2_000_000
    ph = src.generate(n, seed=6)
    plan, bufs = seq.allocate_columns(n)
    status, _ = seq.trace_device(ph, ph, plan, bufs)
    torch.cuda.synchronize()
    assert int(status.item()) == 0
    orders = np.array([0, -3, -6])
    cols = {'order': bufs['order'], 'det_phi': bufs['det_phi'], 'probability': ph.prob}
    res = CaptureResAeff(orders=orders, dispersion_coord='det_phi')(cols)
    R = np.asarray(res['R'], dtype=float)
    assert abs(R[0]) < 0.5
    assert R[2] == pytest.approx(2 * R[1], rel=0.2)
    assert R[1] > 100
    host = {k: v.cpu().numpy() for k, v in cols.items()}
    ref = A.capture_res_aeff(host['order'], host['det_phi'], host['probability'], orders)
    assert np.allclose(R, np.asarray(ref['R'], dtype=float), rtol=1e-9, atol=1e-9)
    assert np.allclose(res['Aeff'], ref['Aeff'], rtol=1e-12)
