"""Pose adjoint on the GPU: the hand-written reverse mode against a float64
torch-autograd restatement and central finite differences.

Spectrometer (200 flat facets, flat detector, 1,207 parameters) with the spot
loss -- RMS cross-dispersion width of the order -5 spot + squared offset of
its dispersion centroid from the nominal position rounded to 1 mm -- and the
CAT array (1000 facets, cylindrical detector, 6,007 parameters) with the mean
resolving power of orders -8..-3 at 0.5 keV.  Bars:
* frozen choices (order sign, normal side, cylinder root) equal the oracle's;
* detector coordinates equal the GPU raytrace at the nominal parameters and
  a fresh raytrace of the moved elements at perturbed parameters (1e-8 mm);
* gradient = torch autograd of the restatement to 1e-8 relative;
* gradient = central differences (h = 1e-4 mm / 1e-6 rad) of the frozen
  float64 forward to 1e-4 relative, per parameter block.
"""
import numpy as np
import pytest
import torch

from oracle import adjoint_torch as AT

pytestmark = pytest.mark.gpu

N_C1 = 200_000
N_C2 = 100_000
C2_ORDERS = [-8, -7, -6, -5, -4, -3, 0]


def _blockwise_rel(a, b, model):
    """max over parameter blocks of max|a - b| / max|b| (blocks with a
    nonzero reference only)."""
    a, b = np.asarray(a), np.asarray(b)
    worst = 0.0
    for key, idx in model.param_slices().items():
        scale = np.max(np.abs(b[idx]))
        if scale > 0:
            worst = max(worst, np.max(np.abs(a[idx] - b[idx])) / scale)
    return worst


@pytest.fixture(scope='module')
def c1():
    from marxs_gb300 import configs
    from marxs_gb300.adjoint import PoseModel, spot_loss
    inst = configs.build('c1')
    host = configs.photons_for('c1', N_C1, seed=41)
    draws = configs.draws_for(inst.draw_slots, N_C1, seed=41)
    model = PoseModel(inst.elements)
    fr, trace = model.trace(host, orders=[-5], draws=draws)
    x_nom = float(torch.round(fr.ref[0, 0]))
    return dict(inst=inst, host=host, draws=draws, model=model, fr=fr, trace=trace,
                loss=spot_loss(x_nom, group=0), prob=fr.torch_dict())


@pytest.fixture(scope='module')
def c2():
    from marxs_gb300 import configs
    from marxs_gb300.adjoint import PoseModel, resolving_power
    inst = configs.build('c2')
    host = configs.annulus_photons(N_C2, 43, inst.aperture_x, energies=np.full(N_C2, 0.5))
    draws = configs.draws_for(inst.draw_slots, N_C2, seed=43)
    model = PoseModel(inst.elements)
    fr, trace = model.trace(host, orders=C2_ORDERS, draws=draws)
    counts = np.bincount(fr.group.cpu().numpy(), minlength=len(C2_ORDERS))
    groups = [g for g, m in enumerate(C2_ORDERS) if m != 0 and counts[g] >= 20]
    assert len(groups) >= 3
    return dict(inst=inst, host=host, draws=draws, model=model, fr=fr, trace=trace,
                loss=resolving_power(C2_ORDERS.index(0), groups), prob=fr.torch_dict())


def _freeze_oracle(case):
    model, prob = case['model'], case['prob']
    flags = model.facet_flags
    from marxs_gb300 import _abi
    cat = torch.from_numpy((flags & _abi.ADJ_FACET_CAT) > 0)
    trans = torch.from_numpy((flags & _abi.ADJ_FACET_TRANSMISSION) > 0)
    return AT.freeze(model.theta0(), prob, cat, trans,
                     phi_lim=(model.det_block[23], model.det_block[24]))


def _traced_xy(case, rows):
    seq, inp, out, bufs = case['trace']
    if 'det_x' in bufs:
        return bufs['det_x'][rows], bufs['det_y'][rows]
    return bufs['det_phi'][rows] * case['model'].det_block[21], bufs['det_y'][rows]


def _random_theta(model, seed, scale=1.0):
    rng = np.random.default_rng(seed)
    th = np.zeros(model.n_params)
    th[0] = model.focallength + 0.5 * scale
    sl = model.param_slices()
    for key, s in (('facet_translation', 0.02), ('facet_rotation', 2e-4),
                   ('detector_translation', 0.05), ('detector_rotation', 5e-4)):
        th[sl[key]] = rng.normal(0, s * scale, len(sl[key]))
    return torch.from_numpy(th).cuda()


@pytest.mark.parametrize('name', ['c1', 'c2'])
def test_frozen_choices_match_the_oracle(name, request):
    case = request.getfixturevalue(name)
    fr = case['fr']
    ref = _freeze_oracle(case)
    assert fr.n > 1000
    np.testing.assert_array_equal(fr.sign.cpu().numpy(), ref['sign'].numpy())
    np.testing.assert_array_equal(fr.nsign.cpu().numpy(), ref['nsign'].numpy())
    if 'root' in ref:
        np.testing.assert_array_equal(fr.root.cpu().numpy(), ref['root'].numpy())


@pytest.mark.parametrize('name', ['c1', 'c2'])
def test_nominal_coordinates_equal_the_raytrace(name, request):
    case = request.getfixturevalue(name)
    fr = case['fr']
    x, y = fr.xy(case['model'].theta0('cuda'))
    tx, ty = _traced_xy(case, fr.rows)
    assert torch.max(torch.abs(x - tx)).item() < 1e-8
    assert torch.max(torch.abs(y - ty)).item() < 1e-8


@pytest.mark.parametrize('name', ['c1', 'c2'])
def test_coordinates_equal_the_torch_restatement(name, request):
    case = request.getfixturevalue(name)
    fr, model = case['fr'], case['model']
    theta = _random_theta(model, 3)
    x, y = fr.xy(theta)
    rx, ry = AT.forward(theta.cpu(), case['prob'])
    np.testing.assert_allclose(x.cpu().numpy(), rx.numpy(), rtol=0, atol=1e-9)
    np.testing.assert_allclose(y.cpu().numpy(), ry.numpy(), rtol=0, atol=1e-9)


@pytest.mark.parametrize('name', ['c1', 'c2'])
def test_perturbed_coordinates_equal_a_raytrace_of_moved_elements(name, request):
    """theta moves the elements the way the raytrace sees them."""
    case = request.getfixturevalue(name)
    fr, model = case['fr'], case['model']
    theta = _random_theta(model, 9)
    try:
        model.apply(theta)
        _, (seq, inp, out, bufs) = model.trace(case['host'], orders=[0], draws=case['draws'],
                                               freeze=False)
    finally:
        model.restore()
    seq0, _, _, bufs0 = case['trace']
    rows = fr.rows
    gr = [s for s in seq.lower().stages if s.id_col is not None][0]
    same = (bufs[gr.id_col][rows] == bufs0[gr.id_col][rows]) & \
        (bufs['order'][rows] == bufs0['order'][rows])
    loc = 'det_x' if 'det_x' in bufs else 'det_phi'
    same &= torch.isfinite(bufs[loc][rows])
    # photons may also switch CAT order sign (p . d changes sign near normal
    # incidence) or cylinder root: choices the frozen forward holds fixed
    from marxs_gb300 import _abi
    flags = model.facet_flags
    moved = AT.freeze(theta.cpu(), case['prob'],
                      torch.from_numpy((flags & _abi.ADJ_FACET_CAT) > 0),
                      torch.from_numpy((flags & _abi.ADJ_FACET_TRANSMISSION) > 0),
                      phi_lim=(model.det_block[23], model.det_block[24]))
    for k in ('sign', 'nsign', 'root'):
        if k in moved:
            same &= (moved[k] == case['prob'][k]).to(same.device)
    assert same.float().mean().item() > 0.9
    x, y = fr.xy(theta)
    if loc == 'det_x':
        tx, ty = bufs['det_x'][rows], bufs['det_y'][rows]
    else:
        tx, ty = bufs['det_phi'][rows] * model.det_block[21], bufs['det_y'][rows]
    assert torch.max(torch.abs(x - tx)[same]).item() < 1e-8
    assert torch.max(torch.abs(y - ty)[same]).item() < 1e-8


@pytest.mark.parametrize('name', ['c1', 'c2'])
def test_gradient_equals_torch_autograd(name, request):
    case = request.getfixturevalue(name)
    fr, model = case['fr'], case['model']
    theta = _random_theta(model, 4, scale=0.5)
    L, g = fr.loss_and_grad(theta, case['loss'])
    prob = dict(case['prob'])
    # the restatement's statistics are two-pass; same loss
    Lr, gr = AT.stats_loss_and_grad(theta.cpu(), prob, fr.n_groups, case['loss'])
    assert abs(float(L) - float(Lr)) <= 1e-9 * abs(float(Lr))
    g, gr = g.cpu().numpy(), gr.numpy()
    assert np.linalg.norm(g - gr) <= 1e-8 * np.linalg.norm(gr)
    assert _blockwise_rel(g, gr, model) <= 1e-7


def test_c1_gradient_equals_central_differences(c1):
    """All 1,207 parameters, h = 1e-4 mm / 1e-6 rad."""
    fr, model = c1['fr'], c1['model']
    theta = model.theta0('cuda')
    _, g = fr.loss_and_grad(theta, c1['loss'])
    fd = fr.finite_differences(theta, c1['loss'])
    g, fd = g.cpu().numpy(), fd.cpu().numpy()
    assert model.n_params == 1207
    assert np.linalg.norm(g - fd) <= 1e-4 * np.linalg.norm(fd)
    assert _blockwise_rel(g, fd, model) <= 1e-4


def test_c2_gradient_equals_central_differences_on_a_subset(c2):
    fr, model = c2['fr'], c2['model']
    theta = model.theta0('cuda')
    _, g = fr.loss_and_grad(theta, c2['loss'])
    busiest = np.argsort(np.bincount(fr.facet.cpu().numpy(), minlength=model.n_facets))[-8:]
    params = np.concatenate([[0], (4 + 6 * busiest[:, None] + np.arange(3)).ravel(),
                             (1 + 6 * busiest[:, None] + np.arange(3)).ravel(),
                             model.n_params - 6 + np.arange(6)])
    fd = fr.finite_differences(theta, c2['loss'], params=params).cpu().numpy()
    g = g.cpu().numpy()[params]
    assert np.linalg.norm(g - fd) <= 1e-4 * np.linalg.norm(fd)
    for blk in (slice(1, 25), slice(25, 49), slice(49, 52), slice(52, 55)):
        assert np.max(np.abs(g[blk] - fd[blk])) <= 1e-4 * np.max(np.abs(fd[blk])), blk


def test_autograd_function_backpropagates_into_theta(c1):
    from marxs_gb300.adjoint import PoseMoments, moment_stats
    fr = c1['fr']
    theta = fr.model.theta0('cuda').requires_grad_(True)
    L = c1['loss'](moment_stats(PoseMoments.apply(theta, fr), fr.ref))
    L.backward()
    _, g = fr.loss_and_grad(theta.detach(), c1['loss'])
    # same kernels; only the order of the atomic sums differs
    assert torch.allclose(theta.grad, g, rtol=1e-10, atol=1e-12 * float(g.abs().max()))


def test_moments_are_deterministic_up_to_summation_order(c1):
    fr = c1['fr']
    th = fr.model.theta0('cuda')
    a, b = fr.moments(th), fr.moments(th)
    assert torch.allclose(a, b, rtol=1e-12, atol=1e-12)


def test_bad_facet_index_is_reported():
    """A facet index outside the table sets the status bit; the host raises."""
    from marxs_gb300 import configs
    from marxs_gb300.adjoint import FrozenPhotons, PoseModel
    inst = configs.build('c1')
    model = PoseModel(inst.elements)
    n = 64
    host = configs.photons_for('c1', n, seed=1)
    dev = torch.device('cuda')
    pos = torch.from_numpy(np.ascontiguousarray(host['pos'][:, :3].T)).to(dev)
    dirs = torch.from_numpy(np.ascontiguousarray(host['dir'][:, :3].T)).to(dev)
    z = torch.zeros(n, dtype=torch.float64, device=dev)
    facet = torch.full((n,), model.n_facets + 3, dtype=torch.int32, device=dev)
    with pytest.raises(ValueError, match='out of range'):
        FrozenPhotons(model, pos, dirs, z + 1.0, z + 1.0, z, z, facet,
                      torch.zeros(n, dtype=torch.int32, device=dev),
                      torch.zeros(n, dtype=torch.int32, device=dev), n_groups=1)


def test_adjoint_is_over_100x_faster_than_finite_differences(c1):
    import time
    fr, model = c1['fr'], c1['model']
    theta = model.theta0('cuda')
    for _ in range(3):
        fr.loss_and_grad(theta, c1['loss'])
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(10):
        _, g = fr.loss_and_grad(theta, c1['loss'])
    torch.cuda.synchronize()
    t_adj = (time.perf_counter() - t0) / 10
    t0 = time.perf_counter()
    fd = fr.finite_differences(theta, c1['loss'])
    torch.cuda.synchronize()
    t_fd = time.perf_counter() - t0
    assert t_fd / t_adj >= 100, (t_fd, t_adj)


def test_graphed_gradient_equals_direct_gradient(c1):
    """The CUDA-graph replay gives the gradient of the current theta."""
    from marxs_gb300.adjoint import GraphedGradient
    fr, model = c1['fr'], c1['model']
    gg = GraphedGradient(fr, c1['loss'])
    for seed in (4, 5):
        theta = _random_theta(model, seed, scale=0.5)
        L, g = gg(theta)
        L0, g0 = fr.loss_and_grad(theta, c1['loss'])
        assert abs(float(L) - float(L0)) <= 1e-12 * abs(float(L0))
        assert torch.allclose(g, g0, rtol=1e-10, atol=1e-12 * float(g0.abs().max()))


class _Precision:
    """The fixture's frozen photons with another moments/gradient precision."""

    def __init__(self, fr, precision):
        self.fr, self.precision = fr, precision

    def __enter__(self):
        self.old = self.fr.precision
        self.fr.precision = self.precision
        return self.fr

    def __exit__(self, *exc):
        self.fr.precision = self.old


def test_fp32local_coordinates_match_float64(c1):
    """FP32-local forward (float-float positions re-centred on every
    element): detector coordinates within 0.1 um RMS / 1 um of float64,
    nominal and perturbed."""
    fr, model = c1['fr'], c1['model']
    for theta in (model.theta0('cuda'), _random_theta(model, 5)):
        x64, y64 = fr.xy(theta)
        with _Precision(fr, 'fp32local'):
            x32, y32 = fr.xy(theta)
        d = torch.cat([x32 - x64, y32 - y64]).cpu().numpy()
        assert np.sqrt(np.mean(d ** 2)) <= 1e-4 and np.max(np.abs(d)) <= 1e-3, \
            (np.sqrt(np.mean(d ** 2)), np.max(np.abs(d)))


def test_fp32local_gradient_equals_central_differences(c1):
    """The FP32-local gradient (float32 reverse sweep, float64 sums) against
    central differences of the float64 forward and against the float64
    adjoint, all 1,207 parameters: 1e-4 relative per parameter block."""
    fr, model = c1['fr'], c1['model']
    theta = model.theta0('cuda')
    _, g64 = fr.loss_and_grad(theta, c1['loss'])
    fd = fr.finite_differences(theta, c1['loss'])
    with _Precision(fr, 'fp32local'):
        _, g32 = fr.loss_and_grad(theta, c1['loss'])
        fd32 = fr.finite_differences(theta, c1['loss'])     # float64 forward either way
    g32, g64, fd, fd32 = (t.cpu().numpy() for t in (g32, g64, fd, fd32))
    # the same float64 forward, up to the atomics' summation order (which the
    # differences amplify to ~1e-8 on the rotations; a float32 forward would
    # be off by ~1e-4)
    assert np.linalg.norm(fd - fd32) <= 1e-6 * np.linalg.norm(fd)
    assert np.linalg.norm(g32 - fd) <= 1e-4 * np.linalg.norm(fd)
    assert _blockwise_rel(g32, fd, model) <= 1e-4
    assert _blockwise_rel(g32, g64, model) <= 1e-4


def test_fp32local_adjoint_needs_a_flat_detector(c2):
    from marxs_gb300.adjoint import PoseModel
    model = PoseModel(c2['inst'].elements)
    with pytest.raises(NotImplementedError):
        model.trace(c2['host'], orders=[-5], draws=c2['draws'], adjoint_precision='fp32local')
