"""The C ABI: header layout agrees with the ctypes mirror; the library loads
and exports every entry point the header declares (no GPU needed)."""
import ctypes
import os
import re
import subprocess

import numpy as np
import pytest

from marxs_gb300 import _abi

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, 'include', 'marxs_gb300.h')

STRUCTS = {
    'mgpu_col': _abi.MgpuCol, 'mgpu_vec': _abi.MgpuVec, 'mgpu_photons': _abi.MgpuPhotons,
    'mgpu_selector': _abi.MgpuSelector, 'mgpu_grid': _abi.MgpuGrid,
    'mgpu_stage': _abi.MgpuStage, 'mgpu_chain': _abi.MgpuChain,
    'mgpu_flat32': _abi.MgpuFlat32, 'mgpu_grid32': _abi.MgpuGrid32, 'mgpu_cyl32': _abi.MgpuCyl32,
    'mgpu_adjoint_problem': _abi.MgpuAdjointProblem, 'mgpu_spline1': _abi.MgpuSpline1,
    'mgpu_source': _abi.MgpuSource, 'mgpu_stats_problem': _abi.MgpuStatsProblem,
    'mgpu_pose_update': _abi.MgpuPoseUpdate,
}


def _c_layout(tmp_path):
    lines = ['#include <stdio.h>', '#include <stddef.h>', '#include "%s"' % HEADER,
             'int main(void) {']
    for cname, cls in STRUCTS.items():
        lines.append('printf("%s size %%zu\\n", sizeof(%s));' % (cname, cname))
        for fname, _ in cls._fields_:
            lines.append('printf("%s.%s %%zu\\n", offsetof(%s, %s));' % (cname, fname, cname, fname))
    lines.append('printf("mgpu_facet size %zu\\n", sizeof(mgpu_facet));')
    for fname in _abi.FACET_DTYPE.names:
        lines.append('printf("mgpu_facet.%s %%zu\\n", offsetof(mgpu_facet, %s));' % (fname, fname))
    lines.append('printf("mgpu_facet32 size %zu\\n", sizeof(mgpu_facet32));')
    for fname in _abi.FACET32_DTYPE.names:
        lines.append('printf("mgpu_facet32.%s %%zu\\n", offsetof(mgpu_facet32, %s));' % (fname, fname))
    lines.append('return 0; }')
    src = tmp_path / 'layout.c'
    src.write_text('\n'.join(lines))
    exe = tmp_path / 'layout'
    subprocess.run(['gcc', '-std=c99', str(src), '-o', str(exe)], check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout
    return dict((k, int(v)) for k, v in (line.rsplit(' ', 1) for line in out.strip().splitlines()))


def test_struct_layout_matches_header(tmp_path):
    c = _c_layout(tmp_path)
    for cname, cls in STRUCTS.items():
        assert c[cname + ' size'] == ctypes.sizeof(cls), cname
        for fname, _ in cls._fields_:
            assert c[cname + '.' + fname] == getattr(cls, fname).offset, (cname, fname)
    assert c['mgpu_facet size'] == _abi.FACET_DTYPE.itemsize
    for fname in _abi.FACET_DTYPE.names:
        assert c['mgpu_facet.' + fname] == _abi.FACET_DTYPE.fields[fname][1], fname
    assert c['mgpu_facet32 size'] == _abi.FACET32_DTYPE.itemsize
    for fname in _abi.FACET32_DTYPE.names:
        assert c['mgpu_facet32.' + fname] == _abi.FACET32_DTYPE.fields[fname][1], fname


def test_header_constants_match():
    text = open(HEADER).read()
    consts = dict(re.findall(r'#define (MGPU_\w+)\s+(0x[0-9a-fA-F]+|\d+)', text))
    assert int(consts['MGPU_ABI_VERSION']) == _abi.MGPU_ABI_VERSION
    assert int(consts['MGPU_MAX_STAGES']) == _abi.MAX_STAGES
    assert int(consts['MGPU_MAX_OUT']) == _abi.MAX_OUT
    for name in ('CHECK_W', 'GENERIC', 'NO_GRID', 'SPLIT_4K'):
        assert int(consts['MGPU_FLAG_' + name], 16) == getattr(_abi, 'FLAG_' + name), name
    for name in ('PROB_RANGE', 'ORDER_EMPTY', 'BAD_STAGE', 'GRID_RANGE', 'GRID_FULL'):
        assert int(consts['MGPU_STATUS_' + name].rstrip('u'), 16) == getattr(_abi, 'STATUS_' + name)
    for name in ('LENS', 'SCATTER', 'FLATDET', 'GRATINGS', 'CYLDET'):
        assert int(consts['MGPU_STAGE_' + name]) == getattr(_abi, 'STAGE_' + name)
    assert int(consts['MGPU_NOALLOC_MAX_CELLS']) == _abi.NOALLOC_MAX_CELLS
    assert int(consts['MGPU_STATUS_ADJ_RANGE'].rstrip('u'), 16) == _abi.STATUS_ADJ_RANGE
    assert int(consts['MGPU_SEL_CDF']) == _abi.SEL_CDF
    assert int(consts['MGPU_SEL_SPLINE']) == _abi.SEL_SPLINE
    for name in ('FREEZE', 'FORWARD', 'BACKWARD', 'DET_FLAT', 'DET_CYL', 'NMOM', 'NSEED',
                 'MAX_GROUPS', 'MAX_FACETS'):
        assert int(consts['MGPU_ADJ_' + name]) == getattr(_abi, 'ADJ_' + name), name
    for name in ('FACET_CAT', 'FACET_TRANSMISSION'):
        assert int(consts['MGPU_ADJ_' + name].rstrip('u'), 16) == getattr(_abi, 'ADJ_' + name)
    for name in ('MAX_GROUPS', 'NRES', 'MEAN', 'MEDIAN', 'STD', 'N_CLIP', 'N_MEMBER', 'AEFF',
                 'N_FINITE', 'ROUNDS'):
        assert int(consts['MGPU_STATS_' + name]) == getattr(_abi, 'STATS_' + name), name
    for name in ('RES_FILTER', 'AEFF_ONLY'):
        assert int(consts['MGPU_STATS_' + name].rstrip('u'), 16) == getattr(_abi, 'STATS_' + name)
    for name in ('ZERO', 'DRAW', 'GIVEN'):
        assert int(consts['MGPU_POSE_' + name]) == getattr(_abi, 'POSE_' + name), name
    for name in ('NONE', 'F64', 'I32', 'I64'):
        assert int(consts['MGPU_ORDER_' + name]) == getattr(_abi, 'ORDER_' + name), name
    assert re.search(r'#define MGPU_ERR_NOALLOC_LIMIT \((-?\d+)\)', text).group(1) == \
        str(_abi.ERR_NOALLOC_LIMIT)


def _declared_functions():
    text = open(HEADER).read()
    return sorted(set(re.findall(r'^\w[\w\s\*]*?\b(mgpu_\w+)\s*\(', text, re.M)))


def test_library_exports_every_declared_symbol():
    if not os.path.exists(_abi.LIB_PATH):
        pytest.skip('library not built')
    lib = ctypes.CDLL(_abi.LIB_PATH)
    declared = _declared_functions()
    assert declared, 'no functions parsed from header'
    for name in declared:
        assert hasattr(lib, name), name
    assert set(declared) == set(_abi.SIGNATURES), 'ctypes signatures out of sync with header'


def test_load_binds_signatures_without_gpu():
    if not os.path.exists(_abi.LIB_PATH):
        pytest.skip('library not built')
    lib = _abi.load()
    assert lib.mgpu_abi_version() == _abi.MGPU_ABI_VERSION


def test_facet_dtype_is_packed_like_c():
    assert _abi.FACET_DTYPE.itemsize % 8 == 0
    a = np.zeros(3, _abi.FACET_DTYPE)
    assert a.nbytes == 3 * _abi.FACET_DTYPE.itemsize


def test_order_guide_table_gives_the_linear_search_result():
    """The guide table (host side of the FP32-local order search) plus forward
    steps reproduces the first index with U < threshold for every row."""
    from marxs_gb300 import configs, lowering
    inst = configs.build('c2')
    sel = lowering.lower_selector(inst.selector)
    th = lowering.selector_thresholds(sel).reshape(sel.cdf.shape)
    guide = lowering.selector_guide(sel)
    assert guide is not None and guide.shape == (th.shape[0], 64)
    rng = np.random.default_rng(0)
    U = np.concatenate([rng.integers(0, 2 ** 53, 20000, dtype=np.uint64),
                        th.ravel(), th.ravel() - np.uint64(1), np.arange(64, dtype=np.uint64) << np.uint64(47)])
    for r in range(0, th.shape[0], 7):
        ref = np.array([np.argmax(np.append(u < th[r], True)) for u in U[:3000]])
        k = guide[r][(U[:3000] >> np.uint64(47)).astype(int)].astype(int)
        for j in range(len(k)):
            while k[j] < th.shape[1] and not (U[j] < th[r][k[j]]):
                k[j] += 1
        assert np.array_equal(k, ref)


def test_entry_points_reject_bad_descriptors_without_a_gpu():
    """Every entry point checks its descriptor on the host and returns
    cudaErrorInvalidValue (1) before any CUDA call, so the checks run here."""
    import ctypes as C
    lib = _abi.load()
    bad = 1
    ph = _abi.MgpuPhotons()
    assert lib.mgpu_trace(None, C.byref(ph), None) == bad
    ch = _abi.MgpuChain()
    ch.n_stages = _abi.MAX_STAGES + 1
    assert lib.mgpu_trace(C.byref(ch), C.byref(ph), None) == bad
    ch.n_stages, ch.precision = 1, 7
    assert lib.mgpu_trace(C.byref(ch), C.byref(ph), None) == bad
    ch.precision, ch.rng = _abi.FP32LOCAL, 9
    assert lib.mgpu_trace(C.byref(ch), C.byref(ph), None) == bad
    ch.rng, ph.n = _abi.RNG_PHILOX, -1
    assert lib.mgpu_trace(C.byref(ch), C.byref(ph), None) == bad
    g = _abi.MgpuGrid()
    assert lib.mgpu_facet_grid_build(None, 0, C.byref(g), None, None, None) == bad
    assert lib.mgpu_facet_grid_build(None, 0, C.byref(g), C.c_void_p(16), C.c_void_p(16),
                                     None) == bad                      # nu = nv = 0
    g.nu = g.nv = 1
    g.cell_start = g.cell_items = 16
    for build in (lambda f, n: lib.mgpu_facet_grid_build(f, n, C.byref(g), C.c_void_p(16),
                                                           C.c_void_p(16), None),
                  lambda f, n: lib.mgpu_facet_grid_build_noalloc(f, n, C.byref(g),
                                                                   C.c_void_p(16), None)):
        assert build(None, 3) == bad                  # facets NULL with n_facets > 0
        assert build(C.c_void_p(16), -1) == bad       # negative facet count
    assert lib.mgpu_plane_intersect(None, 5, _abi.MgpuVec(), _abi.MgpuVec(), None,
                                    _abi.MgpuVec(), _abi.MgpuCol(), _abi.MgpuCol(), None) == bad
    assert lib.mgpu_order_stats(None, None) == bad
    assert lib.mgpu_facet_poses(None, None) == bad
    src = _abi.MgpuSource()
    src.n, src.rng, src.precision = 10, 5, _abi.FP64
    v = _abi.MgpuVec()
    c = _abi.MgpuCol()
    assert lib.mgpu_generate_photons(C.byref(src), v, v, v, c, c, None) == bad
    assert lib.mgpu_pose_adjoint(None, None, 0, None, None, None, None) == bad
    assert lib.mgpu_fma_probe(_abi.FP32LOCAL, 0, 1, None, None) == bad
    assert lib.mgpu_philox4x32_10(None, None, 5, None) == bad
    assert lib.mgpu_philox4x32_10(None, None, -1, None) == bad
