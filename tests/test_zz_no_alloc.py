"""The allocation-free candidate-grid build against the allocating one.

``mgpu_facet_grid_build_noalloc`` exists for callers that cannot allocate
device memory when they rebuild a facet array's candidate grid (a host
whose own pool owns the device memory, or a loop where cudaMalloc/cudaFree
would synchronise the device).  Its scratch is a fixed device array shared
by every call, so these tests call it several times in a row on different
grids and require exactly the output of ``mgpu_facet_grid_build`` (cell
starts and candidate lists are integers: equality is the tolerance) each
time -- a left-over count from the previous call would show up here.

This file is collected last on purpose: it must pass when run alone in a
fresh process (the first call then performs the per-device address lookup)
and after every other test.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _grating_stage(name):
    """Facets of the workload and a candidate grid inside the allocation-free
    entry point's cell limit (2 cells per facet edge)."""
    from marxs_gb300 import configs, _abi
    from marxs_gb300.lowering import grid_params, lower_elements
    inst = configs.build(name)
    st = [s for s in lower_elements(inst.elements) if s.kind == _abi.STAGE_GRATINGS][0]
    g = grid_params(st.facets, cells_per_facet=2.0)
    assert g['nu'] * g['nv'] <= _abi.NOALLOC_MAX_CELLS
    return st.facets, g


def _build(facets, g, noalloc):
    """Run one of the two entry points through the C ABI; the test (the
    caller) owns the output buffers."""
    import torch
    from marxs_gb300 import _abi
    lib = _abi.load()
    dev = torch.device('cuda')
    fac = torch.from_numpy(facets.view(np.uint8).copy()).to(dev)
    ncell = g['nu'] * g['nv']
    start = torch.full((ncell + 1,), -7, dtype=torch.int32, device=dev)
    items = torch.full((g['capacity'],), -7, dtype=torch.int32, device=dev)
    status = torch.zeros(1, dtype=torch.int32, device=dev)
    grid = _abi.MgpuGrid()
    for key in ('o', 'n', 'a', 'b'):
        getattr(grid, key)[:] = [float(x) for x in g[key]]
    grid.u0, grid.v0, grid.cell = g['u0'], g['v0'], g['cell']
    grid.nu, grid.nv = g['nu'], g['nv']
    grid.slope_max, grid.margin = g['slope_max'], g['margin']
    grid.depth[:] = [float(x) for x in g['depth']]
    grid.depth_lip = g['depth_lip']
    grid.cell_start, grid.cell_items = start.data_ptr(), items.data_ptr()
    grid.capacity = g['capacity']
    stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    if noalloc:
        rc = lib.mgpu_facet_grid_build_noalloc(fac.data_ptr(), len(facets), C.byref(grid),
                                               status.data_ptr(), stream)
    else:
        counts = torch.zeros(ncell + 1 + (ncell + 4095) // 4096, dtype=torch.int32, device=dev)
        rc = lib.mgpu_facet_grid_build(fac.data_ptr(), len(facets), C.byref(grid),
                                       counts.data_ptr(), status.data_ptr(), stream)
    assert rc == 0, rc
    torch.cuda.synchronize()
    st = start.cpu().numpy()
    return st, items.cpu().numpy()[:st[-1]], int(status.item())


def test_noalloc_build_matches_allocating_build_on_consecutive_calls():
    # three calls in a row on two different grids: the shared scratch must be
    # cleared by every call
    for name in ('c2', 'c1', 'c2'):
        facets, g = _grating_stage(name)
        ref_start, ref_items, ref_status = _build(facets, g, noalloc=False)
        start, items, status = _build(facets, g, noalloc=True)
        assert ref_status == 0 and status == 0
        assert np.array_equal(start, ref_start), name
        assert np.array_equal(items, ref_items), name
        assert start[-1] > len(facets)          # every facet listed in at least one cell


def test_noalloc_build_rejects_grid_beyond_its_limit():
    from marxs_gb300 import _abi
    facets, g = _grating_stage('c1')
    g = dict(g)
    g['nu'], g['nv'] = _abi.NOALLOC_MAX_CELLS + 1, 1
    import torch
    lib = _abi.load()
    buf = torch.zeros(16, dtype=torch.int32, device='cuda')
    status = torch.zeros(1, dtype=torch.int32, device='cuda')
    grid = _abi.MgpuGrid()
    grid.nu, grid.nv = g['nu'], g['nv']
    grid.cell = g['cell']
    grid.cell_start, grid.cell_items, grid.capacity = buf.data_ptr(), buf.data_ptr(), 16
    rc = lib.mgpu_facet_grid_build_noalloc(None, 0, C.byref(grid), status.data_ptr(),
                                           C.c_void_p(torch.cuda.current_stream().cuda_stream))
    assert rc == _abi.ERR_NOALLOC_LIMIT
    torch.cuda.synchronize()
    assert int(status.item()) == 0


def test_noalloc_build_rejects_bad_facet_arguments():
    """NULL facets with a positive count, or a negative count, are refused
    on the host with cudaErrorInvalidValue (1); nothing is launched."""
    from marxs_gb300 import _abi
    lib = _abi.load()
    grid = _abi.MgpuGrid()
    grid.nu = grid.nv = 1
    grid.cell_start = grid.cell_items = 16
    assert lib.mgpu_facet_grid_build_noalloc(None, 3, C.byref(grid), C.c_void_p(16), None) == 1
    assert lib.mgpu_facet_grid_build_noalloc(C.c_void_p(16), -1, C.byref(grid), C.c_void_p(16),
                                             None) == 1
