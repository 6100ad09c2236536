"""Float64 torch-autograd reference for the pose-gradient (adjoint) kernel.

TEST INFRASTRUCTURE ONLY: tests and the measurement harness use it to check
the hand-written adjoint kernel; the product never imports it.

It restates, vectorised over photons, the frozen-choice forward of the
grating spectrometer (lens -> radial scatter -> facet array -> flat
detector), following the reference formulas:
* PerfectLens direction, marxs/optics/mirror.py:66-71
* RadialMirrorScatter rotations R^T v, marxs/optics/scatter.py:52-67 and
  axangle2mat, marxs/math/rotations.py:50-87
* FinitePlane ray parameter k, marxs/math/geometry.py:233-247
* FlatGrating diffraction, marxs/optics/grating.py:233-266
* FlatDetector local coordinates, marxs/math/geometry.py:249-252
* CircularDetector: Cylinder.intersect, marxs/math/geometry.py:470-564
  (root (-b + root sqrt(b^2 - 4ac)) / 2a), coordinates (phi R, z zoom_z)
Each photon's lens/scatter/detector hit, facet index, order, CAT sign,
normal-side sign, cylinder root and scatter angles are held fixed.

Pose parameters: theta = [f, facet_0 (t_x, t_y, t_z, a_x, a_y, a_z), ...,
facet_{F-1}, detector (6)]; a pose perturbation translates the centre by t
and rotates the element about its centre by R = Rz(a_z) Ry(a_y) Rx(a_x)
(static-frame x, y, z Euler angles, the convention of
marxs/design/uncertainties.py:36-38), applied on top of the base pose.
"""
import torch

ENERGY2WAVE = 1.2398419292004202e-06


def euler_sxyz(a):
    """(..., 3) angles -> (..., 3, 3) matrices Rz(a2) Ry(a1) Rx(a0)."""
    c, s = torch.cos(a), torch.sin(a)
    one, zero = torch.ones_like(a[..., 0]), torch.zeros_like(a[..., 0])
    rx = torch.stack([torch.stack([one, zero, zero], -1),
                      torch.stack([zero, c[..., 0], -s[..., 0]], -1),
                      torch.stack([zero, s[..., 0], c[..., 0]], -1)], -2)
    ry = torch.stack([torch.stack([c[..., 1], zero, s[..., 1]], -1),
                      torch.stack([zero, one, zero], -1),
                      torch.stack([-s[..., 1], zero, c[..., 1]], -1)], -2)
    rz = torch.stack([torch.stack([c[..., 2], -s[..., 2], zero], -1),
                      torch.stack([s[..., 2], c[..., 2], zero], -1),
                      torch.stack([zero, zero, one], -1)], -2)
    return rz @ ry @ rx


def _norm(v):
    return v / torch.sqrt((v * v).sum(-1, keepdim=True))


def _dot(a, b):
    return (a * b).sum(-1)


def _rot_t(axis, angle, v):
    """R^T v for R = axangle2mat(axis, angle)."""
    k = _norm(axis)
    c, s = torch.cos(angle)[..., None], torch.sin(angle)[..., None]
    return c * v - s * torch.cross(k, v, dim=-1) + (1 - c) * _dot(k, v)[..., None] * k


def _front(f, prob):
    """Lens then scatter: position and direction leaving the scatter plane."""
    P0, d0 = prob['P0'], prob['d0']
    # lens: plane crossing (its pose is fixed), then towards the focus
    cL, nL, ezL = prob['lens_c'], prob['lens_n'], prob['lens_ez']
    kL = _dot(cL - P0, nL) / _dot(d0, nL)
    PL = P0 + kL[:, None] * d0
    focus = cL - prob['lens_doff'] * ezL + f * _norm(d0)
    dL = _norm(focus - PL)
    # scatter
    cS, nS = prob['scat_c'], prob['scat_n']
    kS = _dot(cS - PL, nS) / _dot(dL, nS)
    PS = PL + kS[:, None] * dL
    radial = PL - cS
    perp = torch.cross(dL, radial, dim=-1)
    alpha, beta = prob['alpha'], prob['beta']
    d1 = torch.where((alpha != 0)[:, None], _rot_t(perp, alpha, dL), dL)
    dS = torch.where((beta != 0)[:, None], _rot_t(radial, beta, d1), d1)
    return PS, dS


def _facets(theta, prob):
    """Perturbed centre, normal, groove and -perp vectors of each photon's facet."""
    F = prob['facet_c'].shape[0]
    fp = theta[1:1 + 6 * F].reshape(F, 6)
    j = prob['facet']
    R = euler_sxyz(fp[:, 3:6])[j]
    c = prob['facet_c'][j] + fp[j, 0:3]
    n = (R @ prob['facet_n'][j][..., None])[..., 0]
    l = (R @ prob['facet_l'][j][..., None])[..., 0]
    dn = (R @ prob['facet_dneg'][j][..., None])[..., 0]
    return c, n, l, dn


def _grating(PS, dS, c, n, l, dn, sign, nsign, prob):
    kg = _dot(c - PS, n) / _dot(dS, n)
    Pg = PS + kg[:, None] * dS
    p = _norm(dS)
    pl, pd = _dot(p, l), _dot(p, dn)
    pd2 = pd + sign * prob['order'] * ENERGY2WAVE / prob['energy'] / prob['facet_d'][prob['facet']]
    pn2 = torch.sqrt(1.0 - pd2 * pd2 - pl * pl)
    dg = pd2[:, None] * dn + pl[:, None] * l + (nsign * pn2)[:, None] * n
    return Pg, dg


def _cyl_local(theta, Pg, dg, prob):
    F = prob['facet_c'].shape[0]
    dp = theta[1 + 6 * F:7 + 6 * F]
    A = prob['det_Minv'] @ euler_sxyz(dp[3:6]).T
    q = (Pg - (prob['det_c'] + dp[0:3])) @ A.T
    r = dg @ A.T
    a = r[:, 0] ** 2 + r[:, 1] ** 2
    b = 2 * (q[:, 0] * r[:, 0] + q[:, 1] * r[:, 1])
    cc = q[:, 0] ** 2 + q[:, 1] ** 2 - 1
    return q, r, a, b, torch.sqrt(b * b - 4 * a * cc)


def forward(theta, prob):
    """Detector coordinates (x, y) of the frozen photons for parameters theta.

    ``prob`` is a dict of float64 tensors (marxs_gb300.adjoint.FrozenPhotons.torch_dict
    has the keys).
    """
    F = prob['facet_c'].shape[0]
    dp = theta[1 + 6 * F:7 + 6 * F]
    PS, dS = _front(theta[0], prob)
    Pg, dg = _grating(PS, dS, *_facets(theta, prob), prob['sign'], prob['nsign'], prob)
    if prob.get('det_kind', 'flat') == 'cyl':
        q, r, a, b, sd = _cyl_local(theta, Pg, dg, prob)
        s = (-b + prob['root'] * sd) / (2 * a)
        h = q + s[:, None] * r
        return torch.atan2(h[:, 1], h[:, 0]) * prob['det_R'], h[:, 2] * prob['det_zoomz']
    Rd = euler_sxyz(dp[3:6])
    cd = prob['det_c'] + dp[0:3]
    nd, eyd, ezd = Rd @ prob['det_n'], Rd @ prob['det_ey'], Rd @ prob['det_ez']
    kd = _dot(cd - Pg, nd) / _dot(dg, nd)
    Pd = Pg + kd[:, None] * dg
    v = Pd - cd
    return _dot(v, eyd), _dot(v, ezd)


def freeze(theta, prob, cat, transmission, phi_lim=None):
    """Order sign, normal side (and cylinder root) of every photon at theta.

    cat / transmission: per-facet booleans.  Sign: -1 for FlatGrating
    (grating.py:145-172), sign(p . d) with 0 -> +1 for CATGrating
    (grating.py:291-302); side: sign(p . n), negated for reflection gratings
    (grating.py:262-264).  Root: the smaller non-negative parameter among the
    roots inside the cylinder's z and phi range (geometry.py:519-540),
    phi_lim = reduced (b1, b2) borders.
    """
    with torch.no_grad():
        PS, dS = _front(theta[0], prob)
        c, n, l, dn = _facets(theta, prob)
        p = _norm(dS)
        j = prob['facet']
        sign = torch.where(cat[j], torch.where(_dot(p, dn) < 0, -1.0, 1.0),
                           torch.full_like(p[:, 0], -1.0))
        nsign = torch.sign(_dot(p, n)) * torch.where(transmission[j], 1.0, -1.0)
        out = {'sign': sign, 'nsign': nsign}
        if prob.get('det_kind', 'flat') == 'cyl':
            Pg, dg = _grating(PS, dS, c, n, l, dn, sign, nsign, prob)
            q, r, a, b, sd = _cyl_local(theta, Pg, dg, prob)
            hits = []
            for root in (1.0, -1.0):
                s = (-b + root * sd) / (2 * a)
                h = q + s[:, None] * r
                phi = torch.remainder(torch.atan2(h[:, 1], h[:, 0]), 2 * torch.pi)
                b1, b2 = phi_lim
                inside = ((b1 <= phi) & (phi <= b2)) if b1 < b2 else ((b1 <= phi) | (phi <= b2))
                hits.append(((s >= 0) & (h[:, 2].abs() <= 1) & inside, s))
            (h1, s1), (h2, s2) = hits
            out['root'] = torch.where(h2 & ~(h1 & (s2 >= s1)), -1.0, 1.0)
        return out


def spot_loss(x, y, w, x_nom):
    """RMS cross-dispersion width + squared centroid offset (weights w)."""
    W = w.sum()
    mx = (w * x).sum() / W
    my = (w * y).sum() / W
    sig = torch.sqrt((w * (y - my) ** 2).sum() / W)
    return sig + (mx - x_nom) ** 2


def group_stats(x, y, w, group, n_groups):
    """Weighted centroid and variance of (x, y) per group (two-pass)."""
    out = {k: [] for k in ('W', 'mean_x', 'mean_y', 'var_x', 'var_y')}
    for g in range(n_groups):
        m = group == g
        wg, xg, yg = w[m], x[m], y[m]
        W = wg.sum()
        mx, my = (wg * xg).sum() / W, (wg * yg).sum() / W
        out['W'].append(W)
        out['mean_x'].append(mx)
        out['mean_y'].append(my)
        out['var_x'].append((wg * (xg - mx) ** 2).sum() / W)
        out['var_y'].append((wg * (yg - my) ** 2).sum() / W)
    return {k: torch.stack(v) for k, v in out.items()}


def stats_loss_and_grad(theta, prob, n_groups, loss_fn):
    """loss_fn(group_stats) and its gradient by torch autograd."""
    th = theta.clone().detach().requires_grad_(True)
    x, y = forward(th, prob)
    L = loss_fn(group_stats(x, y, prob['w'], prob['group'], n_groups))
    (g,) = torch.autograd.grad(L, th)
    return L.detach(), g


def loss_and_grad(theta, prob, x_nom):
    th = theta.clone().detach().requires_grad_(True)
    x, y = forward(th, prob)
    L = spot_loss(x, y, prob['w'], x_nom)
    (g,) = torch.autograd.grad(L, th)
    return L.detach(), g
