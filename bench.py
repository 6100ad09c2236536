#!/usr/bin/env python
"""Photon-raytrace throughput of the GB300 backend on the CAT-grating workload.

Workload (one "step" = one pass of the element chain over one batch):
1e8 photons per GPU through a PerfectLens (f = 12 m), RadialMirrorScatter
(5", 1"), a Parallel of 1000 CATGrating facets on a Rowland torus
(R = r = 5900 mm, EfficiencyFile-style 64 x 15 order table, nearest-hit grid
lookup) and a CircularDetector (R = 5900 mm); Philox in-kernel randomness.
Photons are synthetic (seeded annulus aperture, piecewise-linear spectrum).

Usage: ``python bench.py [--gpus N --steps K --warmup W --impl native|reference]``.
Prints one JSON line on rank 0.  ``value`` is device-resident throughput
(inputs already in HBM); ``e2e`` is the same metric through the public
``GpuSequence(...)(table)`` call with pinned host buffers, host<->device
copies included.  ``--impl reference`` times the CPU oracle (the reference
algorithm restated in numpy) on all host cores on a bounded sample.

Sub-lines of the same JSON line (each can be switched off by a --no-* flag):
``fp32local_*`` / ``fp64_*`` and ``um_error`` (the two precisions and the
FP32-local error against float64), ``roofline`` (the chain kernel against
the measured HBM copy bandwidth), ``e2e``, ``source_pipeline`` (photons
generated on the device, event columns to the host), ``analysis``
(CaptureResAeff on the device columns), ``cat_stack`` (CATL1L2Stack facets),
``stages`` (each stage alone, against HBM and the measured FMA peaks),
``adjoint`` and ``design`` (pose gradients, design loop), ``tolerancing``
and ``cpu_baseline`` (the oracle on one core).
"""
import argparse
import json
import math
import os
import subprocess
import sys
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = 'photons/s at 1e8 (FP32-local vs FP64); adjoint grads/s vs finite-diff; µm err'
UNIT = 'photons/s'
WORKLOAD = 'cat_rowland_1000facets_circular_detector'

# DRAM bytes (read + write) per photon of each chain kernel, from one ncu
# capture (dram__bytes_read.sum + dram__bytes_write.sum) of a 4e6-photon
# launch, scaled to the launch by photon count
NCU_TRAFFIC_BYTES_PER_PHOTON = {'fp64': (358.2e6 + 735.3e6) / 4e6,
                                'fp32local': (355.7e6 + 724.0e6) / 4e6}


def parse():
    p = argparse.ArgumentParser()
    p.add_argument('--gpus', type=int, default=1)
    p.add_argument('--steps', type=int, default=10)
    p.add_argument('--warmup', type=int, default=3)
    p.add_argument('--impl', default='native', choices=['native', 'reference'])
    p.add_argument('--photons', type=float, default=1e8, help='photons per GPU per step')
    p.add_argument('--precision', default='auto', choices=['auto', 'fp64', 'fp32local'])
    p.add_argument('--no-e2e', action='store_true')
    p.add_argument('--no-cpu', action='store_true')
    p.add_argument('--e2e-steps', type=int, default=3)
    p.add_argument('--no-adjoint', action='store_true')
    p.add_argument('--adjoint-photons', type=float, default=1e6)
    p.add_argument('--no-design', action='store_true')
    p.add_argument('--design-photons', type=float, default=1e7)
    p.add_argument('--design-steps', type=int, default=50)
    p.add_argument('--no-tolerancing', action='store_true')
    p.add_argument('--tolerancing-photons', type=float, default=1e7)
    p.add_argument('--tolerancing-sets', type=int, default=10)
    p.add_argument('--no-stages', action='store_true')
    p.add_argument('--stage-photons', type=float, default=2e7)
    return p.parse_args()


def peaks():
    path = os.path.join(ROOT, 'MEASURED_PEAKS.json')
    try:
        with open(path) as f:
            d = json.load(f)
        return float(d['hbm_gbs']), 'measured'
    except (OSError, KeyError, ValueError):
        return 6800.0, 'fallback'


# ---------------------------------------------------------------- clocks
class ClockSampler:
    FIELDS = ('index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,'
              'clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,'
              'clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap')

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.path = os.path.join('/tmp', 'mgpu_clocks_%d_%d.csv' % (os.getpid(), index))

    def start(self):
        try:
            self.f = open(self.path, 'w')
            self.proc = subprocess.Popen(['nvidia-smi', '-i', str(self.index),
                                          '--query-gpu=' + self.FIELDS, '--format=csv,noheader',
                                          '-lms', '100'], stdout=self.f,
                                         stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return {'sm_mhz': None, 'sm_max_mhz': None, 'reasons': ['nvidia-smi unavailable']}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.f.close()
        sm, mx, reasons = [], [], set()
        names = ['hw_slowdown', 'hw_thermal_slowdown', 'sw_thermal_slowdown', 'sw_power_cap']
        with open(self.path) as f:
            for line in f:
                parts = [x.strip() for x in line.split(',')]
                if len(parts) < 9:
                    continue
                try:
                    sm.append(float(parts[1].split()[0]))
                    mx.append(float(parts[2].split()[0]))
                except ValueError:
                    continue
                for name, val in zip(names, parts[5:9]):
                    if val.lower().startswith('active'):
                        reasons.add(name)
        os.unlink(self.path)
        sm.sort()
        return {'sm_mhz': sm[len(sm) // 2] if sm else None, 'sm_max_mhz': max(mx) if mx else None,
                'reasons': sorted(reasons), 'samples': len(sm)}


# ---------------------------------------------------------------- CPU legs
def _oracle_chunk(args):
    n, seed, row0 = args
    sys.path.insert(0, ROOT)
    from marxs_gb300 import configs
    from oracle.raytrace import run_sequence
    inst = configs.build('c2')
    ph = configs.photons_for('c2', n, seed=seed)
    dr = configs.draws_for(inst.draw_slots, n, seed=seed)
    t = time.perf_counter()
    run_sequence(inst.elements, ph, dr)
    return time.perf_counter() - t


def cpu_baseline_single(target_s=12.0):
    """Single-process oracle on a bounded C2 sample (rank 0, N = 1)."""
    t_small = _oracle_chunk((4000, 101, 0))
    n = int(min(200000, max(4000, 4000 * target_s / max(t_small, 1e-3))))
    dt = _oracle_chunk((n, 102, 0))
    return {'value': n / dt, 'unit': UNIT, 'cores': 1, 'kind': 'port',
            'sample': '%d photons of the same workload (1000 facets), one process, '
                      'float64 numpy oracle with pre-drawn randomness' % n}


_REF_WORKER = {}


def _ref_worker_init(barrier):
    _REF_WORKER['barrier'] = barrier


def _ref_worker_steps(args):
    """One pool process of the reference arm: builds the instrument once,
    then per step makes its photon sample and draws (untimed), waits at the
    barrier for every other process and times only the raytrace."""
    n, seed0, n_steps = args
    sys.path.insert(0, ROOT)
    from marxs_gb300 import configs
    from oracle.raytrace import run_sequence
    inst = configs.build('c2')
    out = []
    for step in range(n_steps):
        ph = configs.photons_for('c2', n, seed=seed0 + step)
        dr = configs.draws_for(inst.draw_slots, n, seed=seed0 + step)
        _REF_WORKER['barrier'].wait(timeout=900)
        t = time.perf_counter()
        run_sequence(inst.elements, ph, dr)
        out.append(time.perf_counter() - t)
    return out


def run_reference(args):
    """--impl reference: the CPU oracle on all host cores, bounded sample per
    step.  One process per core; each step every process traces its own
    photons, all starting together at a barrier; the step time is the
    slowest process's raytrace time (instrument set-up, photon and draw
    generation are outside the timed region)."""
    import multiprocessing as mp
    rank = int(os.environ.get('RANK', '0'))
    if rank != 0:
        return 0
    cores = len(os.sched_getaffinity(0))
    per_worker = 30000
    ctx = mp.get_context('spawn')
    n_steps = args.warmup + args.steps
    barrier = ctx.Barrier(cores)
    with ctx.Pool(cores, initializer=_ref_worker_init, initargs=(barrier,)) as pool:
        per = pool.map(_ref_worker_steps,
                       [(per_worker, 1000 + 97 * w, n_steps) for w in range(cores)], chunksize=1)
    times = [max(p[k] for p in per) for k in range(args.warmup, n_steps)]
    step_s = sum(times) / len(times)
    value = per_worker * cores / step_s
    line = {'metric': METRIC, 'value': value, 'unit': UNIT, 'impl': 'reference',
            'n_gpus': args.gpus, 'steps': args.steps, 'warmup': args.warmup,
            'ms_per_step': step_s * 1e3, 'higher_is_better': True, 'scaling': 'weak',
            'vs_baseline': None, 'dtype': 'f64', 'data': 'synthetic',
            'config': {'workload': WORKLOAD, 'photons_per_step': per_worker * cores,
                       'n_facets': 1000},
            'cpu_baseline': {'value': value, 'unit': UNIT, 'cores': cores, 'kind': 'port',
                             'sample': '%d photons per step (%d per process, all processes '
                                       'starting together; set-up and photon generation '
                                       'untimed) of the same workload, float64 numpy oracle'
                                       % (per_worker * cores, per_worker)},
            'e2e': {'value': value, 'unit': UNIT, 'h2d_bytes_per_step': 0,
                    'd2h_bytes_per_step': 0}}
    print(json.dumps(line), flush=True)
    return 0


# ---------------------------------------------------------------- GPU leg
def algorithmic_bytes(seq):
    """Bytes per photon: input state read once (pos, dir, pol 3x8 each,
    energy 8, probability 8 = 88), final state written once (pos, dir, pol,
    probability = 80), every stage column written once at its dtype."""
    cols, draws = seq.column_bytes()
    return 88 + 80 + cols + draws


def precision_error(a, b, torch):
    """Detector-position error of FP32-local against float64, same photons and
    draws, over photons whose facet and order agree (micron)."""
    fa, fb = a['bufs']['facet'], b['bufs']['facet']
    oa, ob = a['bufs']['order'], b['bufs']['order']
    agree = (fa == fb) & ((oa == ob) | (torch.isnan(oa) & torch.isnan(ob)))
    # a CAT sign decision sign(p . d) taken within a few float32 roundings of
    # zero (blaze < 2e-7 rad) is a discrete flip like a facet-edge flip
    agree &= ~((b['bufs']['blaze'] < 2e-7) & (ob != 0))
    pa, pb = a['out'].pos, b['out'].pos
    m = agree & torch.isfinite(pb).all(0) & torch.isfinite(b['bufs']['det_phi'])
    d = ((pa - pb) ** 2).sum(0).sqrt()[m] * 1e3
    dphi = ((a['bufs']['det_phi'] - b['bufs']['det_phi']).abs() * 5900.0)[m] * 1e3
    dy = (a['bufs']['det_y'] - b['bufs']['det_y']).abs()[m] * 1e3
    out = {'photons_compared': int(m.sum()), 'decision_mismatch': int((~agree).sum()),
           'pos_rms_um': float((d ** 2).mean().sqrt()), 'pos_max_um': float(d.max()),
           'det_phi_R_rms_um': float((dphi ** 2).mean().sqrt()), 'det_phi_R_max_um': float(dphi.max()),
           'det_y_rms_um': float((dy ** 2).mean().sqrt()), 'det_y_max_um': float(dy.max())}
    # every other float column over the agreeing photons: local coordinates
    # (mm -> um), detector pixels (x 0.024 mm pixel -> um), angles (rad)
    cols = {}
    for name, kind in (('mirror_x', 'mm'), ('mirror_y', 'mm'), ('grat_y', 'mm'), ('grat_z', 'mm'),
                       ('detpix_x', 'pix'), ('detpix_y', 'pix'), ('blaze', 'rad'),
                       ('inplanescatter', 'rad'), ('perpplanescatter', 'rad')):
        if name not in a['bufs'] or name not in b['bufs']:
            continue
        x, y = a['bufs'][name], b['bufs'][name]
        k = agree & torch.isfinite(y)
        e = (x - y).abs()[k]
        if kind == 'mm':
            e = e * 1e3
        elif kind == 'pix':
            e = e * 0.024e3
        key = name + ('_um' if kind != 'rad' else '_rad')
        cols[key] = {'rms': float((e ** 2).mean().sqrt()), 'max': float(e.max())}
    out['columns'] = cols
    return out


def source_pipeline_bench(args, torch, inst, n, head, row_base, dist):
    """Photons made on the GPU (point source, RandomArbitraryPdf spectrum on
    the workload's 200 energy knots, unpolarized, through a CircleAperture
    annulus r in [300, 500] mm), traced, and the detector event columns
    (det_phi, det_y, order, facet) copied to pinned host memory: no photon
    list crosses the host link."""
    import numpy as np
    from marxs_gb300 import configs
    from marxs_gb300.gpu import DevicePhotons, GpuSequence
    from marxs_gb300.source import CircleAperture, DeviceSource, simulate_events
    from marxs_gb300.sharding import max_over_ranks
    knots, dens = configs.spectrum_knots(2)
    ap = CircleAperture(position=[12000., 0, 0], zoom=[1, 500, 500], r_inner=300.)
    src = DeviceSource(ap, energy={'energy': knots, 'fluxdensity': dens}, precision=head)
    seq = GpuSequence(elements=inst.elements, precision=head, rng='philox', seed=12345)
    cols = ['det_phi', 'det_y', 'order', 'facet']
    out = simulate_events(src, seq, n, cols, seed=7, row_base=row_base)
    d2h = sum(out[k].numel() * out[k].element_size() for k in cols)
    times = []
    for step in range(1 + args.e2e_steps):
        torch.cuda.synchronize()
        t = time.perf_counter()
        simulate_events(src, seq, n, cols, seed=7 + step, row_base=row_base, out=out)
        if step > 0:
            times.append(time.perf_counter() - t)
    s = max_over_ranks([sum(times) / len(times)], dist, device='cuda')[0]
    world = dist.get_world_size() if dist is not None else 1
    return {'value': world * n / s, 'unit': UNIT, 'ms_per_step': s * 1e3,
            'h2d_bytes_per_step': 0, 'd2h_bytes_per_step': d2h,
            'source_precision': head,
            'api': 'simulate_events(DeviceSource(CircleAperture, spectrum), GpuSequence): '
                   'generate + trace + event columns to pinned host memory, chunks of 8e6 '
                   'on two streams'}


def analysis_bench(args, torch, rr, n):
    """CaptureResAeff (orders -10..10, det_phi) over the event columns the
    timed trace left on the device: the per-order effective area and
    sigma-clipped resolving power, one mgpu_order_stats call per step; the
    oracle on a 1e6-photon host sample of the same columns beside it."""
    import numpy as np
    from marxs_gb300.analysis import CaptureResAeff
    from oracle import analysis as A
    bufs, out = rr['bufs'], rr['out']
    cols = {'order': bufs['order'], 'det_phi': bufs['det_phi'], 'probability': out.prob}
    cap = CaptureResAeff(orders=np.arange(-10, 11), dispersion_coord='det_phi')
    res = cap(cols)
    stream = torch.cuda.current_stream()
    times = []
    for _ in range(3):
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        res = cap(cols)
        b.record(stream)
        torch.cuda.synchronize()
        times.append(a.elapsed_time(b))
    ms = min(times)
    m = min(n, 1_000_000)
    host = {k: v[:m].cpu().numpy() for k, v in cols.items()}
    t = time.perf_counter()
    A.capture_res_aeff(host['order'], host['det_phi'], host['probability'], np.arange(-10, 11))
    cpu_s = time.perf_counter() - t
    return {'value': n / (ms / 1e3), 'unit': 'photons/s', 'ms_per_call': ms,
            'orders': 21, 'Rgrat': float(res['Rgrat']),
            'bytes_read_per_photon': 24,
            'cpu_baseline': {'value': m / cpu_s, 'unit': 'photons/s', 'cores': 1, 'kind': 'port',
                             'sample': '%d photons of the same columns, numpy oracle' % m},
            'api': 'CaptureResAeff(orders=-10..10, dispersion_coord="det_phi")(device columns)'}


def tolerancing_bench(args, torch):
    """run_tolerances over facet wiggles of the 1000-facet CAT array
    (sigma 0.5 mm / 1 arcmin per axis, a new realisation per parameter set),
    1e7 photons at 0.5 keV generated once on the device, FP32-local trace,
    CaptureResAeff (orders -8..0, det_phi) per set: device poses against the
    same loop with the wiggle applied on the host (Parallel.generate_elements,
    lowering and upload of the facet tables, grid build)."""
    import numpy as np
    from marxs_gb300 import configs, geomath
    from marxs_gb300.analysis import CaptureResAeff
    from marxs_gb300.gpu import DevicePhotons, GpuSequence
    from marxs_gb300.source import CircleAperture, DeviceSource
    from marxs_gb300.tolerancing import DeviceFacetPoses, run_tolerances, wiggle
    n = int(args.tolerancing_photons)
    K = int(args.tolerancing_sets)
    arcmin = np.deg2rad(1. / 60)
    params = [{'dx': 0.5, 'dy': 0.5, 'dz': 0.5, 'rx': arcmin, 'ry': arcmin, 'rz': arcmin}] * K
    inst = configs.build('c2')
    seq = GpuSequence(elements=inst.elements, precision='fp32local', rng='philox', seed=21)
    poses = DeviceFacetPoses(seq, inst.gas, seed=3)
    ap = CircleAperture(position=[12000., 0, 0], zoom=[1, 500, 500], r_inner=300.)
    photons = DeviceSource(ap, energy=0.5).generate(n, seed=9)
    cap = CaptureResAeff(orders=np.arange(-8, 1), dispersion_coord='det_phi')
    run_tolerances(photons, seq, wiggle, poses, params[:2], cap)
    torch.cuda.synchronize()
    t = time.perf_counter()
    res = run_tolerances(photons, seq, wiggle, poses, params, cap)
    torch.cuda.synchronize()
    dev_s = (time.perf_counter() - t) / K
    # host wiggle: new elem_uncertainty, generate_elements, relower, trace, analyse
    rng = np.random.default_rng(0)
    F = len(inst.gas.elements)
    plan, bufs = seq.allocate_columns(n)
    out = DevicePhotons(n)
    host_s = []
    for k in range(3):
        torch.cuda.synchronize()
        t = time.perf_counter()
        tr = rng.normal(0, 0.5, (F, 3))
        rot = rng.normal(0, arcmin, (F, 3))
        inst.gas.elem_uncertainty = [geomath.compose(a, geomath.euler2mat(*b, 'sxyz'), np.ones(3))
                                     for a, b in zip(tr, rot)]
        inst.gas.generate_elements()
        hseq = GpuSequence(elements=inst.elements, precision='fp32local', rng='philox', seed=21)
        plan, bufs = hseq.allocate_columns(n)
        hseq.trace_device(photons, out, plan, bufs)
        cap(dict(bufs, probability=out.prob))
        torch.cuda.synchronize()
        host_s.append(time.perf_counter() - t)
    host = float(np.median(host_s))
    return {'value': 1.0 / dev_s, 'unit': 'parameter sets/s', 's_per_set': dev_s,
            'photons_per_set': n, 'sets': K, 'host_pose_s_per_set': host,
            'speedup_vs_host_poses': host / dev_s,
            'Rgrat_first_last': [float(res[0]['Rgrat']), float(res[-1]['Rgrat'])],
            'api': 'run_tolerances(DevicePhotons, GpuSequence, wiggle, DeviceFacetPoses, params, '
                   'CaptureResAeff)'}


def cat_stack_bench(args, torch, dev_in, n, row_base):
    """The Arcus-style chain: the same photons through lens, scatter, 1000
    CATL1L2Stack facets (membrane, quality factor, L1 grating/support, L2
    absorption and diffraction), catsupportbars and the circular detector,
    FP32-local, Philox; CUDA events per step."""
    from marxs_gb300 import configs
    from marxs_gb300.gpu import DevicePhotons, GpuSequence
    inst = configs.build('c6')
    seq = GpuSequence(elements=inst.elements, precision='fp32local', rng='philox', seed=12345)
    out = DevicePhotons(n)
    plan, bufs = seq.allocate_columns(n)
    stream = torch.cuda.current_stream()
    for _ in range(2):
        seq.trace_device(dev_in, out, plan, bufs, row_base=row_base)
    torch.cuda.synchronize()
    # steps queued back to back (the host's per-call check overlaps the
    # previous step), CUDA events around the block
    steps = 3
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    a.record(stream)
    for _ in range(steps):
        status, _ = seq.trace_device(dev_in, out, plan, bufs, row_base=row_base)
    b.record(stream)
    torch.cuda.synchronize()
    if int(status.item()):
        raise RuntimeError('cat stack trace status 0x%x' % int(status.item()))
    ms = a.elapsed_time(b) / steps
    hit = float((bufs['facet'] >= 0).float().mean().item())
    del out, plan, bufs
    torch.cuda.empty_cache()
    return {'value': n / (ms / 1e3), 'unit': 'photons/s', 'ms_per_step': ms,
            'precision': 'fp32local', 'facet_hit_fraction': hit,
            'workload': 'c2 photons through 1000 CATL1L2Stack facets + catsupportbars'}


def fma_peaks(torch):
    """Measured FMA throughput (flop/s) of the FP32 and FP64 pipes: the
    library's FMA-chain probe, 8 blocks of 256 threads per SM."""
    import ctypes as C
    from marxs_gb300 import _abi
    lib = _abi.load()
    sms = torch.cuda.get_device_properties(0).multi_processor_count
    blocks = sms * 8
    out = {}
    for name, prec, iters, dt in (('fp32', _abi.FP32LOCAL, 1 << 16, torch.float32),
                                  ('fp64', _abi.FP64, 1 << 10, torch.float64)):
        buf = torch.empty(blocks * 256, dtype=dt, device='cuda')
        stream = torch.cuda.current_stream()

        def run():
            _abi.check(lib.mgpu_fma_probe(prec, blocks, iters, C.c_void_p(buf.data_ptr()),
                                          C.c_void_p(stream.cuda_stream)), 'mgpu_fma_probe')
        for _ in range(3):
            run()
        ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
              for _ in range(5)]
        for a, b in ev:
            a.record(stream)
            run()
            b.record(stream)
        torch.cuda.synchronize()
        ms = sorted(a.elapsed_time(b) for a, b in ev)[2]
        out[name] = 2.0 * 8 * iters * 256 * blocks / (ms / 1e3)
    return out


def grid_candidates(torch, seq, ph):
    """Mean candidate-list length per photon at the facet stage's grid
    lookup (the lookup's own arithmetic on the photons entering the stage;
    0 outside the grid or beyond its slope limit)."""
    from marxs_gb300 import _abi
    low = seq.lower()
    si = [k for k, st in enumerate(low.stages) if st.kind == _abi.STAGE_GRATINGS][0]
    g = low.stages[si].grid
    start = low.stage_grid_bufs[si][0].to(torch.int64)
    vec = lambda x: torch.tensor([float(v) for v in x], dtype=torch.float64, device='cuda')[:, None]
    o, nrm, a, b = vec(g['o']), vec(g['n']), vec(g['a']), vec(g['b'])
    rel = ph.pos - o
    dn = (ph.dir * nrm).sum(0)
    da = (ph.dir * a).sum(0)
    db = (ph.dir * b).sum(0)
    t0 = -(rel * nrm).sum(0) / dn
    u = (rel * a).sum(0) + t0 * da
    v = (rel * b).sum(0) + t0 * db
    iu = torch.floor((u - g['u0']) / g['cell'])
    iv = torch.floor((v - g['v0']) / g['cell'])
    ok = ((iu >= 0) & (iu < g['nu']) & (iv >= 0) & (iv < g['nv']) &
          (da.abs() <= g['slope_max'] * dn.abs()) & (db.abs() <= g['slope_max'] * dn.abs()))
    cell = (iu.clamp(0, g['nu'] - 1) * g['nv'] + iv.clamp(0, g['nv'] - 1)).to(torch.int64)
    cnt = (start[cell + 1].clamp(max=g['capacity']) - start[cell]).clamp(min=0)
    return float((cnt * ok).sum()) / ph.n


def stages_bench(args, torch, inst, dev_in):
    """Each stage of the workload's chain launched on its own (a one-stage
    chain, generic kernel) on the photons the previous stages produced:
    its own algorithmic bytes (state read 88 B, state written 80 B, its
    columns) against the measured HBM peak, and for the facet stage the
    intersect arithmetic against the measured FMA peak (per photon: 37 flops
    per grid candidate, 153 per hit for diffraction and transport)."""
    from marxs_gb300 import _abi
    from marxs_gb300.gpu import DevicePhotons, GpuSequence
    n = min(int(args.stage_photons), dev_in.n)
    hbm, hbm_src = peaks()
    fma = fma_peaks(torch)
    src = dev_in
    if n < dev_in.n:
        src = DevicePhotons(n)
        for k in ('pos', 'dir', 'pol'):
            getattr(src, k).copy_(getattr(dev_in, k)[:, :n])
        src.energy.copy_(dev_in.energy[:n])
        src.prob.copy_(dev_in.prob[:n])
    names = ['lens', 'scatter', 'facets', 'detector']
    res = {'photons': n, 'fma_peak_flops': fma, 'hbm_peak_gbs': hbm, 'hbm_peak_source': hbm_src,
           'kernel': 'chain kernels, generic one-stage chain'}
    for prec in ('fp32local', 'fp64'):
        cur = src
        rows = {}
        for k, elem in enumerate(inst.elements):
            seq = GpuSequence(elements=[elem], precision=prec, rng='philox', seed=12345)
            plan, bufs = seq.allocate_columns(n)
            out = DevicePhotons(n)
            hits = torch.zeros(_abi.MAX_STAGES, dtype=torch.int64, device='cuda')
            seq.trace_device(cur, out, plan, bufs, hits=hits)
            torch.cuda.synchronize()
            n_hit = int(hits[0])
            stream = torch.cuda.current_stream()
            for _ in range(2):
                seq.trace_device(cur, out, plan, bufs)
            torch.cuda.synchronize()
            reps = 5              # back to back: the host work overlaps the launches
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(stream)
            for _ in range(reps):
                seq.trace_device(cur, out, plan, bufs)
            b.record(stream)
            torch.cuda.synchronize()
            ms = a.elapsed_time(b) / reps
            B = algorithmic_bytes(seq)
            gbs = B * n / (ms / 1e3) / 1e9
            row = {'ms': ms, 'bytes_per_photon': B, 'achieved_gbs': gbs, 'hbm_frac': gbs / hbm,
                   'hits': n_hit}
            if names[k] == 'facets':
                cand = grid_candidates(torch, seq, cur)
                flops = 37.0 * cand * n + 153.0 * n_hit
                rate = flops / (ms / 1e3)
                peak = fma['fp32' if prec == 'fp32local' else 'fp64']
                row.update({'candidates_per_photon': cand, 'flops': flops, 'flop_rate': rate,
                            'fma_frac': rate / peak,
                            'fma_pipe': 'fp32' if prec == 'fp32local' else 'fp64'})
            rows[names[k]] = row
            del plan, bufs
            if cur is not src:
                del cur
            cur = out
        res[prec] = rows
    del cur
    torch.cuda.empty_cache()
    return res


def adjoint_bench(args, torch):
    """Pose gradients on the 200-facet spectrometer: hand-written adjoint vs
    central finite differences (h = 1e-4 mm / 1e-6 rad) over all 1,207
    parameters.  Loss: RMS cross-dispersion width of the order -5 spot +
    squared offset of its dispersion centroid from the nominal position
    (rounded to 1 mm).  Orders and scatter angles come from one FP32-local
    Philox trace of the photons and are then held fixed."""
    import numpy as np
    from marxs_gb300 import configs
    from marxs_gb300.adjoint import PoseModel, spot_loss
    from marxs_gb300.gpu import DevicePhotons, GpuSequence
    n = int(args.adjoint_photons)
    inst = configs.build('c1')
    host = configs.photons_for('c1', n, seed=3)
    model = PoseModel(inst.elements)
    fr, _ = model.trace(host, orders=[-5], precision='fp32local', rng='philox', seed=3)
    loss = spot_loss(float(torch.round(fr.ref[0, 0])), group=0)
    theta = model.theta0('cuda')
    stream = torch.cuda.current_stream()
    for _ in range(5):
        fr.loss_and_grad(theta, loss)
    K = 20
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(2)]
    torch.cuda.synchronize()
    ev[0].record(stream)
    for _ in range(K):
        L, g = fr.loss_and_grad(theta, loss)
    ev[1].record(stream)
    torch.cuda.synchronize()
    grad_ms = ev[0].elapsed_time(ev[1]) / K
    from marxs_gb300.adjoint import GraphedGradient
    gg = GraphedGradient(fr, loss)
    for _ in range(5):
        gg(theta)
    torch.cuda.synchronize()
    ev[0].record(stream)
    for _ in range(K):
        Lg, gg_grad = gg(theta)
    ev[1].record(stream)
    torch.cuda.synchronize()
    graph_ms = ev[0].elapsed_time(ev[1]) / K
    fr.finite_differences(theta, loss, params=np.arange(16))        # warm
    torch.cuda.synchronize()
    ev[0].record(stream)
    fd = fr.finite_differences(theta, loss)
    ev[1].record(stream)
    torch.cuda.synchronize()
    fd_ms = ev[0].elapsed_time(ev[1])
    g_np, fd_np = g.cpu().numpy(), fd.cpu().numpy()

    def blockwise(a):
        worst = 0.0
        for idx in model.param_slices().values():
            sc = np.max(np.abs(fd_np[idx]))
            if sc > 0:
                worst = max(worst, float(np.max(np.abs(a[idx] - fd_np[idx])) / sc))
        return worst
    blk = blockwise(g_np)
    # the same gradient with FP32-local moments and reverse sweep
    fr.precision = 'fp32local'
    for _ in range(5):
        fr.loss_and_grad(theta, loss)
    torch.cuda.synchronize()
    ev[0].record(stream)
    for _ in range(K):
        _, g32 = fr.loss_and_grad(theta, loss)
    ev[1].record(stream)
    torch.cuda.synchronize()
    grad32_ms = ev[0].elapsed_time(ev[1]) / K
    gg32 = GraphedGradient(fr, loss)
    for _ in range(5):
        gg32(theta)
    torch.cuda.synchronize()
    ev[0].record(stream)
    for _ in range(K):
        gg32(theta)
    ev[1].record(stream)
    torch.cuda.synchronize()
    graph32_ms = ev[0].elapsed_time(ev[1]) / K
    fr.precision = 'fp64'
    g32_np = g32.cpu().numpy()
    fp32local = {'grad_ms': graph32_ms, 'grads_per_s': 1e3 / graph32_ms,
                 'grad_eager_ms': grad32_ms, 'speedup_vs_fd': fd_ms / graph32_ms,
                 'rel_err_vs_fd': float(np.linalg.norm(g32_np - fd_np) / np.linalg.norm(fd_np)),
                 'blockwise_rel_err_vs_fd': blockwise(g32_np),
                 'note': 'moments and reverse sweep in FP32-local precision (float-float '
                         'positions re-centred on every element, float32 reverse sweep, '
                         'float64 sums), against the same float64 central differences'}
    # one forward pass of the plain FP64 raytrace over the same photons, with
    # the orders and scatter angles fixed (pre-drawn): the forward a
    # raytrace-based finite difference repeats 2 x 1,207 times
    draws = configs.draws_for(inst.draw_slots, n, seed=3)
    seq = GpuSequence(inst.elements, precision='fp64', rng='predrawn')
    dev_in = DevicePhotons.from_columns(host)
    dev_out = DevicePhotons(n)
    plan, bufs = seq.allocate_columns(n)
    draws_dev = seq._draws_to_device(seq.lower(), draws, n)
    for _ in range(3):
        seq.trace_device(dev_in, dev_out, plan, bufs, draws=draws_dev)
    torch.cuda.synchronize()
    ev[0].record(stream)
    for _ in range(5):
        seq.trace_device(dev_in, dev_out, plan, bufs, draws=draws_dev)
    ev[1].record(stream)
    torch.cuda.synchronize()
    trace_ms = ev[0].elapsed_time(ev[1]) / 5
    fd_trace_ms = 2 * model.n_params * trace_ms
    return {
        'workload': 'spectrometer_200facets_flat_detector: order -5 spot loss, '
                    '%d parameters' % model.n_params,
        'photons_traced': n, 'photons_in_loss': fr.n, 'params': model.n_params,
        'dtype': 'f64', 'grad_ms': graph_ms, 'grads_per_s': 1e3 / graph_ms,
        'grad_eager_ms': grad_ms,
        'fd_ms': fd_ms, 'fd_launches': 2 * model.n_params,
        'speedup_vs_fd': fd_ms / graph_ms, 'speedup_vs_fd_eager': fd_ms / grad_ms,
        'fd_raytrace_ms': fd_trace_ms, 'raytrace_fp64_ms_per_pass': trace_ms,
        'speedup_vs_fd_raytrace': fd_trace_ms / graph_ms,
        'rel_err_vs_fd': float(np.linalg.norm(g_np - fd_np) / np.linalg.norm(fd_np)),
        'blockwise_rel_err_vs_fd': blk, 'loss': float(L), 'fp32local': fp32local,
        'grad_note': 'grad_ms: forward + torch loss + reverse captured in one CUDA graph '
                     '(GraphedGradient); grad_eager_ms: the same launched op by op',
        'fd_note': 'fd_ms: central differences on the frozen float64 forward kernel '
                   '(2 x params launches); fd_raytrace_ms: 2 x params x one measured FP64 '
                   'raytrace pass of all traced photons with pre-drawn randomness'}


def design_bench(args, torch):
    """Adam on the 1000 CAT facet tilts and the detector pose (3,006
    parameters), maximising the mean resolving power of orders -8..-3 at
    0.5 keV; every step re-traces the photons (FP32-local, fresh Philox
    draws), freezes the trace and takes the gradient through the adjoint."""
    import numpy as np
    from marxs_gb300 import configs
    from marxs_gb300.adjoint import PoseModel, design_loop, moment_stats, resolving_power
    from marxs_gb300.gpu import DevicePhotons, GpuSequence
    orders = [-8, -7, -6, -5, -4, -3]
    n = int(args.design_photons)
    inst = configs.build('c2')
    host = configs.annulus_photons(n, 5, inst.aperture_x, energies=np.full(n, 0.5))
    photons = DevicePhotons.from_columns(host)
    del host
    model = PoseModel(inst.elements)
    torch.cuda.reset_peak_memory_stats()
    base = torch.cuda.memory_allocated()
    res = design_loop(model, photons, orders, steps=args.design_steps, seed=1000)
    hist = res['history']
    step_s = [h['seconds'] for h in hist[1:]] or [hist[0]['seconds']]

    def evaluate(theta, seed=4242):
        try:
            model.apply(theta)
            fr, _ = model.trace(photons, orders + [0], precision='fp32local', rng='philox',
                                seed=seed, theta=theta)
        finally:
            model.restore()
        cnt = torch.bincount(fr.group.long(), minlength=len(orders) + 1).cpu().numpy()
        groups = [g for g in range(len(orders)) if cnt[g] >= 20]
        return fr, float(resolving_power(len(orders), groups)(moment_stats(fr.moments(theta),
                                                                           fr.ref))), groups

    th0 = model.theta0('cuda')
    _, r0, _ = evaluate(th0)
    fr, r1, groups = evaluate(res['theta'])
    # finite differences of the same loss on the frozen float64 forward: time a
    # subset of the optimised parameters and scale to all of them
    sl = model.param_slices()
    opt_idx = np.concatenate([sl['facet_rotation'], sl['detector_translation'],
                              sl['detector_rotation']])
    loss = resolving_power(len(orders), groups)
    sub = opt_idx[:: max(1, len(opt_idx) // 64)]
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(2)]
    stream = torch.cuda.current_stream()
    fr.finite_differences(res['theta'], loss, params=sub[:4])
    torch.cuda.synchronize()
    ev[0].record(stream)
    fr.finite_differences(res['theta'], loss, params=sub)
    ev[1].record(stream)
    torch.cuda.synchronize()
    fd_s = ev[0].elapsed_time(ev[1]) / 1e3 * len(opt_idx) / len(sub)
    # the same sampled parameters from the adjoint: the speed-up is quoted
    # at the accuracy the comparison shows
    fd = fr.finite_differences(res['theta'], loss, params=sub)
    _, g_adj = fr.loss_and_grad(res['theta'], loss)
    g_sub = g_adj[torch.from_numpy(sub).to(g_adj.device)]
    rel_err = float(torch.linalg.norm(g_sub - fd) / torch.linalg.norm(fd))
    for _ in range(2):
        fr.loss_and_grad(res['theta'], loss)
    torch.cuda.synchronize()
    ev[0].record(stream)
    for _ in range(5):
        fr.loss_and_grad(res['theta'], loss)
    ev[1].record(stream)
    torch.cuda.synchronize()
    grad_s = ev[0].elapsed_time(ev[1]) / 1e3 / 5
    seq = GpuSequence(inst.elements, precision='fp64', rng='philox', seed=1)
    out = DevicePhotons(n)
    plan, bufs = seq.allocate_columns(n)
    for _ in range(2):
        seq.trace_device(photons, out, plan, bufs)
    torch.cuda.synchronize()
    ev[0].record(stream)
    for _ in range(3):
        seq.trace_device(photons, out, plan, bufs)
    ev[1].record(stream)
    torch.cuda.synchronize()
    trace_s = ev[0].elapsed_time(ev[1]) / 1e3 / 3
    return {
        'workload': 'cat_rowland_1000facets_circular_detector at 0.5 keV: mean resolving '
                    'power of orders -8..-3, Adam over facet tilts + detector pose',
        'photons_per_step': n, 'steps': len(hist), 'params_optimised': int(len(opt_idx)),
        'seconds_per_step': float(np.mean(step_s)),
        'resolving_power_nominal': r0, 'resolving_power_final': r1,
        'resolving_power_history': [round(h['resolving_power'], 3) for h in hist],
        'photons_in_loss': fr.n, 'gradient_s': grad_s,
        'fd_frozen_s_per_gradient': fd_s, 'fd_frozen_sample_params': int(len(sub)),
        'rel_err_vs_fd': rel_err,
        'fd_raytrace_fp64_s_per_gradient': 2 * len(opt_idx) * trace_s,
        'raytrace_fp64_s_per_pass': trace_s,
        'speedup_vs_fd_frozen': fd_s / grad_s,
        'speedup_vs_fd_raytrace': 2 * len(opt_idx) * trace_s / grad_s,
        'peak_device_bytes_above_inputs': int(max(h['peak_bytes'] for h in hist) - base),
        'note': 'seconds_per_step includes the re-trace, lowering of the moved facets, '
                'freeze, forward and backward; gradient_s is forward + backward of the '
                'adjoint alone; fd_frozen scales a timed subset of the parameters; '
                'rel_err_vs_fd compares the adjoint with those central differences '
                '(h = 1e-4 mm / 1e-6 rad) on the same subset'}


def main():
    args = parse()
    if args.impl == 'reference':
        return run_reference(args)
    import numpy as np
    import torch
    from marxs_gb300 import configs
    from marxs_gb300.gpu import GpuSequence, DevicePhotons, pinned_photons
    from marxs_gb300 import _abi
    from marxs_gb300.sharding import weak_shard, max_over_ranks

    world = int(os.environ.get('WORLD_SIZE', '1'))
    rank = int(os.environ.get('RANK', '0'))
    local = int(os.environ.get('LOCAL_RANK', '0'))
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group('nccl', device_id=torch.device('cuda', local))

    def barrier():
        if dist is not None:
            dist.barrier()
        torch.cuda.synchronize()

    n = int(args.photons)
    inst = configs.build('c2')
    host = configs.photons_for('c2', n, seed=2 + 7919 * rank)
    dev_in = DevicePhotons.from_columns(host)
    row_base = weak_shard(rank, n)[0]      # Philox streams keyed by global photon id

    modes = []
    if args.precision in ('auto', 'fp32local'):
        modes.append('fp32local')
    if args.precision in ('auto', 'fp64'):
        modes.append('fp64')

    results = {}
    for mode in modes:
        seq = GpuSequence(elements=inst.elements, precision=mode, rng='philox', seed=12345)
        dev_out = DevicePhotons(n)
        plan, bufs = seq.allocate_columns(n)
        status = torch.zeros(1, dtype=torch.int32, device='cuda')
        hits = torch.zeros(_abi.MAX_STAGES, dtype=torch.int64, device='cuda')
        try:
            seq.trace_device(dev_in, dev_out, plan, bufs, status=status, hits=hits,
                             row_base=row_base)
            torch.cuda.synchronize()
        except RuntimeError as exc:
            if args.precision == 'auto':
                results[mode] = {'error': str(exc)}
                continue
            raise
        stream = torch.cuda.current_stream()
        for _ in range(args.warmup):
            seq.trace_device(dev_in, dev_out, plan, bufs, status=status, hits=hits,
                             row_base=row_base)
        barrier()
        clocks = ClockSampler(local)
        clocks.start()
        time.sleep(0.3)
        ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
              for _ in range(args.steps)]
        barrier()
        t0 = time.perf_counter()
        for k in range(args.steps):
            ev[k][0].record(stream)
            seq.trace_device(dev_in, dev_out, plan, bufs, status=status, hits=hits,
                             row_base=row_base)
            ev[k][1].record(stream)
        barrier()
        wall = time.perf_counter() - t0
        ck = clocks.stop()
        code = int(status.item())
        if code:
            raise RuntimeError('kernel status 0x%x' % code)
        step_ms = [a.elapsed_time(b) for a, b in ev]
        mean_ms = sum(step_ms) / len(step_ms)
        tot_ms = wall * 1e3
        tot_ms, mean_ms = max_over_ranks([tot_ms, mean_ms], dist, device='cuda')
        results[mode] = {'seq': seq, 'plan': plan, 'bufs': bufs, 'out': dev_out, 'mean_ms': mean_ms,
                         'wall_ms': tot_ms, 'clocks': ck,
                         'photons_per_s': world * n * args.steps / (tot_ms / 1e3),
                         'kernel_photons_per_s': n / (mean_ms / 1e3),
                         'hits': hits.cpu().tolist()}

    ok_modes = [m for m in modes if 'seq' in results.get(m, {})]
    head = ok_modes[0]
    r = results[head]
    seq = r['seq']
    hbm, hbm_src = peaks()
    B = algorithmic_bytes(seq)
    achieved = B * n / (r['mean_ms'] / 1e3) / 1e9
    traffic = NCU_TRAFFIC_BYTES_PER_PHOTON.get(head)
    line = {
        'metric': METRIC, 'value': r['photons_per_s'], 'unit': UNIT, 'n_gpus': world,
        'steps': args.steps, 'warmup': args.warmup, 'ms_per_step': r['wall_ms'] / args.steps,
        'higher_is_better': True, 'scaling': 'weak', 'vs_baseline': None,
        'dtype': 'f32' if head == 'fp32local' else 'f64', 'io_dtype': 'f64',
        'data': 'synthetic (seeded annulus aperture, piecewise-linear spectrum, seeded '
                'facet jitter)',
        'config': {'workload': WORKLOAD, 'photons_per_gpu': n, 'n_facets': len(inst.gas.elements),
                   'precision': head, 'rng': 'philox', 'layout': 'SoA float64 planes',
                   'l2': 'inputs (%.1f GB) larger than L2 (129 MB)' % (dev_in.nbytes() / 1e9)},
        'roofline': {'bound': 'hbm', 'achieved': achieved, 'peak': hbm, 'unit': 'GB/s',
                     'frac': achieved / hbm, 'peak_source': hbm_src,
                     'bytes_per_photon': B,
                     'traffic': None if traffic is None else traffic * n,
                     'kernel': 'chain_%s_kernel' % head},
        'gpu_launches': args.steps,
        'clocks': r['clocks'],
    }
    for m in modes:
        rr = results.get(m, {})
        if 'seq' in rr:
            line['%s_photons_per_s' % m] = rr['photons_per_s']
            line['%s_ms_per_step' % m] = rr['mean_ms']
        elif rr:
            line['%s_error' % m] = rr.get('error')
    if 'fp32local' in ok_modes and 'fp64' in ok_modes:
        line['fp32local_over_fp64'] = (results['fp32local']['photons_per_s'] /
                                       results['fp64']['photons_per_s'])
        line['um_error'] = precision_error(results['fp32local'], results['fp64'], torch)

    # end to end through the public table call, pinned host buffers
    if not args.no_e2e:
        e2e_n = n
        pristine = pinned_photons(e2e_n)
        for k in pristine.colnames:
            np.copyto(pristine[k], host[k][:e2e_n])
        work = pinned_photons(e2e_n)
        seq_e = GpuSequence(elements=inst.elements, precision=head, rng='philox', seed=12345)
        times = []
        h2d = d2h = 0
        for step in range(1 + args.e2e_steps):
            for k in pristine.colnames:
                torch.from_numpy(work[k]).copy_(torch.from_numpy(pristine[k]))
            for k in list(work.colnames):
                if k not in pristine.colnames:
                    work.remove_column(k)
            barrier()
            t = time.perf_counter()
            seq_e(work, row_base=row_base)
            torch.cuda.synchronize()
            dt = time.perf_counter() - t
            if step > 0:
                times.append(dt)
        h2d = sum(work[k].nbytes for k in pristine.colnames)
        d2h = sum(work[k].nbytes for k in work.colnames if k not in ('energy',))
        e2e_s = sum(times) / len(times)
        e2e_s = max_over_ranks([e2e_s], dist, device='cuda')[0]
        line['e2e'] = {'value': world * e2e_n / e2e_s, 'unit': UNIT, 'h2d_bytes_per_step': h2d,
                       'd2h_bytes_per_step': d2h, 'ms_per_step': e2e_s * 1e3,
                       'api': 'GpuSequence(elements)(PhotonTable) with pinned host columns'}
    if not args.no_e2e:
        line['source_pipeline'] = source_pipeline_bench(args, torch, inst, n, head, row_base, dist)
    if rank == 0 and world == 1:
        line['analysis'] = analysis_bench(args, torch, results[head], n)
    if rank == 0 and world == 1 and head == 'fp32local':
        for k in ('seq', 'plan', 'bufs', 'out'):
            for rr in results.values():
                rr.pop(k, None)
        torch.cuda.empty_cache()
        line['cat_stack'] = cat_stack_bench(args, torch, dev_in, n, row_base)
    if rank == 0 and world == 1 and not args.no_stages:
        for k in ('seq', 'plan', 'bufs', 'out'):
            for rr in results.values():
                rr.pop(k, None)
        torch.cuda.empty_cache()
        line['stages'] = stages_bench(args, torch, inst, dev_in)
    if rank == 0 and world == 1 and not args.no_adjoint:
        for k in ('seq', 'plan', 'bufs', 'out'):
            for rr in results.values():
                rr.pop(k, None)
        torch.cuda.empty_cache()
        line['adjoint'] = adjoint_bench(args, torch)
    if rank == 0 and world == 1 and not args.no_design:
        line['design'] = design_bench(args, torch)
    if rank == 0 and world == 1 and not args.no_tolerancing:
        line['tolerancing'] = tolerancing_bench(args, torch)
    if rank == 0 and world == 1 and not args.no_cpu:
        line['cpu_baseline'] = cpu_baseline_single()
    if rank == 0:
        print(json.dumps(line), flush=True)
    if dist is not None:
        dist.destroy_process_group()
    return 0


if __name__ == '__main__':
    sys.exit(main())
