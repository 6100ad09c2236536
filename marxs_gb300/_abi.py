"""ctypes mirror of ``include/marxs_gb300.h`` and the library loader.

The structures here must match the C header byte for byte; a CPU test
compiles the header with the system C compiler and compares every size and
field offset.  Loading fails loudly when the library has not been built:
there is no CPU fallback for any of the entry points.
"""
import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, 'libmarxs_gb300.so')

MGPU_ABI_VERSION = 3
MAX_STAGES = 16
MAX_OUT = 10
FACET_CYL = 34
MAX_DRAWS = 6

STATUS_PROB_RANGE = 0x1
STATUS_ORDER_EMPTY = 0x2
STATUS_BAD_STAGE = 0x4
STATUS_GRID_RANGE = 0x8
STATUS_GRID_FULL = 0x10
STATUS_BAD_W = 0x20
STATUS_TABLE_RANGE = 0x80
FLAG_CHECK_W = 0x1
FLAG_GENERIC = 0x2
FLAG_NO_GRID = 0x4
FLAG_SPLIT_4K = 0x8

NOALLOC_MAX_CELLS = 65536
ERR_NOALLOC_LIMIT = -2
STATUS_ADJ_RANGE = 0x40
SEL_CDF, SEL_SPLINE = 0, 1
ADJ_FREEZE, ADJ_FORWARD, ADJ_BACKWARD = 0, 1, 2
ADJ_DET_FLAT, ADJ_DET_CYL = 0, 1
ADJ_NMOM = 5
ADJ_NSEED = 4
ADJ_MAX_GROUPS = 64
ADJ_MAX_FACETS = 4096
ADJ_FACET_CAT = 0x1
ADJ_FACET_TRANSMISSION = 0x2

FP64 = 0
FP32LOCAL = 1
RNG_PREDRAWN = 0
RNG_PHILOX = 1

STAGE_LENS = 1
STAGE_SCATTER = 2
STAGE_FLATDET = 3
STAGE_GRATINGS = 4
STAGE_CYLDET = 5
STAGE_SUPPORT = 6
STAGE_DETARRAY = 7
# stages that search a table of plane elements through a candidate grid
FACET_STAGES = (4, 7)


class MgpuCol(C.Structure):
    _fields_ = [('ptr', C.c_void_p), ('stride', C.c_int64)]


class MgpuVec(C.Structure):
    _fields_ = [('ptr', C.c_void_p), ('stride', C.c_int64), ('cstride', C.c_int64)]


class MgpuPhotons(C.Structure):
    _fields_ = [('n', C.c_int64),
                ('pos', MgpuVec), ('dir', MgpuVec), ('pol', MgpuVec),
                ('energy', MgpuCol), ('prob', MgpuCol),
                ('pos_out', MgpuVec), ('dir_out', MgpuVec), ('pol_out', MgpuVec),
                ('prob_out', MgpuCol)]


class MgpuSpline1(C.Structure):
    _fields_ = [('nx', C.c_int32), ('ny', C.c_int32), ('n_surf', C.c_int32), ('pad', C.c_int32),
                ('tx', C.c_void_p), ('ty', C.c_void_p), ('c', C.c_void_p), ('c32', C.c_void_p),
                ('tx_ff', C.c_void_p), ('ty_ff', C.c_void_p)]


class MgpuSelector(C.Structure):
    _fields_ = [('n_rows', C.c_int32), ('n_orders', C.c_int32), ('by_energy', C.c_int32),
                ('sorted', C.c_int32), ('energy', C.c_void_p), ('cdf', C.c_void_p),
                ('total', C.c_void_p), ('orders', C.c_void_p), ('thresholds', C.c_void_p),
                ('kind', C.c_int32), ('pad', C.c_int32), ('spline', MgpuSpline1),
                ('guide', C.c_void_p), ('e_mid', C.c_void_p), ('e0_f', C.c_float),
                ('e_scale_f', C.c_float)]


class MgpuFlat32(C.Structure):
    _fields_ = [('c_hi', C.c_float * 3), ('c_lo', C.c_float * 3), ('ex', C.c_float * 3),
                ('ey', C.c_float * 3), ('ez', C.c_float * 3), ('hy', C.c_float),
                ('hz', C.c_float), ('p', C.c_float * 6)]


class MgpuGrid32(C.Structure):
    _fields_ = [('o_hi', C.c_float * 3), ('o_lo', C.c_float * 3), ('n', C.c_float * 3),
                ('a', C.c_float * 3), ('b', C.c_float * 3), ('u0', C.c_float),
                ('v0', C.c_float), ('inv_cell', C.c_float), ('slope_max', C.c_float),
                ('nu', C.c_int32), ('nv', C.c_int32), ('depth', C.c_float * 6)]


class MgpuCyl32(C.Structure):
    _fields_ = [('c_hi', C.c_float * 3), ('c_lo', C.c_float * 3), ('e1', C.c_float * 3),
                ('e2', C.c_float * 3), ('a', C.c_float * 3), ('R', C.c_float),
                ('Rz', C.c_float), ('w1', C.c_float * 2), ('w2', C.c_float * 2),
                ('arc', C.c_int32), ('rpix_hi', C.c_float), ('rpix_lo', C.c_float),
                ('inv_pix', C.c_float), ('cp0', C.c_float), ('cp1', C.c_float),
                ('k0', C.c_int32), ('nk', C.c_int32)]


class MgpuGrid(C.Structure):
    _fields_ = [('o', C.c_double * 3), ('n', C.c_double * 3), ('a', C.c_double * 3),
                ('b', C.c_double * 3), ('u0', C.c_double), ('v0', C.c_double),
                ('cell', C.c_double), ('nu', C.c_int32), ('nv', C.c_int32),
                ('slope_max', C.c_double), ('margin', C.c_double),
                ('depth', C.c_double * 6), ('depth_lip', C.c_double),
                ('cell_start', C.c_void_p), ('cell_items', C.c_void_p),
                ('capacity', C.c_int32), ('pad', C.c_int32)]


class MgpuCatStack(C.Structure):
    _fields_ = [('blaze_center', C.c_double), ('d_blaze_mm', C.c_double), ('qf', C.c_double),
                ('l1_open', C.c_double), ('l1_d', C.c_double), ('l1_vec', C.c_void_p),
                ('l1_selector', C.c_int32), ('l1_n_trans', C.c_int32), ('l1_trans_e', C.c_void_p),
                ('l1_trans_t', C.c_void_p), ('l2_open', C.c_double), ('l2_shadow', C.c_double),
                ('l2_total', C.c_double), ('l2_inner', C.c_double), ('l1_vec32', C.c_void_p),
                ('l1_wd_hi', C.c_float), ('l1_wd_lo', C.c_float), ('qf32', C.c_float),
                ('l2_open32', C.c_float), ('l2_absorb32', C.c_float), ('l2_inv_inner32', C.c_float),
                ('blaze_center32', C.c_float), ('d_blaze32', C.c_float),
                ('l1_open_u53', C.c_int64), ('l1_trans_e32', C.c_void_p),
                ('l1_trans_t32', C.c_void_p)]


class MgpuStage(C.Structure):
    _fields_ = [('kind', C.c_int32), ('id_num', C.c_int32), ('first_writer', C.c_int32),
                ('n_facets', C.c_int32), ('frame', C.c_double * 14), ('cyl', C.c_double * 32),
                ('p', C.c_double * 8), ('out', MgpuCol * MAX_OUT), ('id_out', C.c_void_p),
                ('id_stride', C.c_int64), ('draw', C.c_void_p * MAX_DRAWS),
                ('draw_stride', C.c_int64),
                ('facets', C.c_void_p), ('selectors', C.c_void_p), ('n_selectors', C.c_int32),
                ('facet_sel0', C.c_int32), ('grid', MgpuGrid), ('aux_size', C.c_int32),
                ('pad2', C.c_int32), ('aux32', C.c_uint8 * 128),
                ('facets32', C.c_void_p), ('table', C.c_void_p),
                ('spline', MgpuSpline1), ('stack', C.c_void_p), ('sel0', MgpuSelector),
                ('grating_d', MgpuCol), ('blaze_add', MgpuCol), ('facet_cyl', C.c_void_p)]


class MgpuChain(C.Structure):
    _fields_ = [('n_stages', C.c_int32), ('precision', C.c_int32), ('rng', C.c_int32),
                ('flags', C.c_uint32), ('seed', C.c_uint64), ('row_base', C.c_uint64),
                ('status', C.c_void_p),
                ('hits', C.c_void_p), ('stages', MgpuStage * MAX_STAGES)]


# facet record as a numpy structured dtype (C layout of mgpu_facet)
FACET_DTYPE = np.dtype([('c', '<f8', 3), ('ex', '<f8', 3), ('ey', '<f8', 3), ('ez', '<f8', 3),
                        ('hy', '<f8'), ('hz', '<f8'), ('l', '<f8', 3), ('dneg', '<f8', 3),
                        ('dgrat', '<f8'), ('id_num', '<i4'), ('selector', '<i4'),
                        ('cat', '<i4'), ('transmission', '<i4')], align=True)

FACET32_DTYPE = np.dtype([('c_hi', '<f4', 3), ('hy', '<f4'), ('c_lo', '<f4', 3), ('hz', '<f4'),
                          ('ex', '<f4', 3), ('ey', '<f4', 3), ('ez', '<f4', 3),
                          ('l', '<f4', 3), ('dneg', '<f4', 3), ('wd_hi', '<f4'), ('wd_lo', '<f4'),
                          ('id_num', '<i4'), ('selector', '<i4'), ('flags', '<i4'),
                          ('pad', '<i4', 4)], align=True)
assert FACET32_DTYPE.itemsize == 128

# name -> (restype, argtypes) of every exported entry point
class MgpuSource(C.Structure):
    _fields_ = [('n', C.c_int64), ('seed', C.c_uint64), ('row_base', C.c_uint64),
                ('rng', C.c_int32), ('n_bins', C.c_int32), ('energy', C.c_double),
                ('e_x', C.c_void_p), ('e_width', C.c_void_p), ('e_cdf', C.c_void_p),
                ('e_index', C.c_void_p), ('pol_random', C.c_int32), ('precision', C.c_int32),
                ('pol_angle', C.c_double), ('dir', C.c_double * 3), ('pol_v1', C.c_double * 3),
                ('pol_v2', C.c_double * 3), ('center', C.c_double * 3), ('v_y', C.c_double * 3),
                ('v_z', C.c_double * 3), ('phi0', C.c_double), ('phi1', C.c_double),
                ('r_inner2', C.c_double), ('prob', C.c_double), ('draws', C.c_void_p),
                ('e_lo_ff', C.c_void_p), ('e_width_f', C.c_void_p), ('e_thresh', C.c_void_p)]


class MgpuAdjointProblem(C.Structure):
    _fields_ = [('n', C.c_int64), ('n_facets', C.c_int32), ('n_groups', C.c_int32),
                ('det_kind', C.c_int32), ('precision', C.c_int32),
                ('pos', C.c_void_p), ('dir', C.c_void_p), ('alpha', C.c_void_p),
                ('beta', C.c_void_p), ('energy', C.c_void_p), ('weight', C.c_void_p),
                ('facet', C.c_void_p), ('order', C.c_void_p), ('group', C.c_void_p),
                ('sign', C.c_void_p), ('nsign', C.c_void_p), ('root', C.c_void_p),
                ('lens', C.c_double * 10), ('scatter', C.c_double * 6),
                ('facets', C.c_void_p), ('facet_flags', C.c_void_p),
                ('det', C.c_double * 32), ('ref', C.c_void_p), ('x_out', C.c_void_p),
                ('y_out', C.c_void_p), ('rot', C.c_void_p), ('status', C.c_void_p)]


STATS_MAX_GROUPS = 64
STATS_NRES = 8
STATS_MEAN, STATS_MEDIAN, STATS_STD, STATS_N_CLIP = 0, 1, 2, 3
STATS_N_MEMBER, STATS_AEFF, STATS_N_FINITE, STATS_ROUNDS = 4, 5, 6, 7
ORDER_NONE, ORDER_F64, ORDER_I32, ORDER_I64 = 0, 1, 2, 3
STATS_RES_FILTER = 0x1
STATS_AEFF_ONLY = 0x2


class MgpuStatsProblem(C.Structure):
    _fields_ = [('n', C.c_int64), ('value', MgpuCol), ('order', C.c_void_p),
                ('order_stride', C.c_int64), ('order_type', C.c_int32), ('n_groups', C.c_int32),
                ('prob', MgpuCol), ('aeff_mask', C.c_void_p), ('flags', C.c_uint32),
                ('maxiters', C.c_int32), ('sigma', C.c_double),
                ('orders', C.c_double * STATS_MAX_GROUPS), ('work', C.c_void_p),
                ('work_bytes', C.c_int64), ('result', C.c_void_p)]


POSE_ZERO, POSE_DRAW, POSE_GIVEN = 0, 1, 2


class MgpuPoseUpdate(C.Structure):
    _fields_ = [('n_facets', C.c_int32), ('mode', C.c_int32), ('seed', C.c_uint64),
                ('sigma', C.c_double * 6), ('offset', C.c_double * 6), ('given', C.c_void_p),
                ('perturb_out', C.c_void_p), ('outer', C.c_double * 16), ('local', C.c_void_p),
                ('groove', C.c_void_p), ('facets', C.c_void_p), ('facets32', C.c_void_p)]


SIGNATURES = {
    'mgpu_abi_version': (C.c_int, []),
    'mgpu_device_sm_count': (C.c_int, []),
    'mgpu_trace': (C.c_int, [C.POINTER(MgpuChain), C.POINTER(MgpuPhotons), C.c_void_p]),
    'mgpu_facet_grid_build': (C.c_int, [C.c_void_p, C.c_int32, C.POINTER(MgpuGrid), C.c_void_p,
                                        C.c_void_p, C.c_void_p]),
    'mgpu_facet_grid_build_noalloc': (C.c_int, [C.c_void_p, C.c_int32, C.POINTER(MgpuGrid),
                                                C.c_void_p, C.c_void_p]),
    'mgpu_plane_intersect': (C.c_int, [C.c_void_p, C.c_int64, MgpuVec, MgpuVec, C.c_void_p,
                                       MgpuVec, MgpuCol, MgpuCol, C.c_void_p]),
    'mgpu_cylinder_intersect': (C.c_int, [C.c_void_p, C.c_int64, MgpuVec, MgpuVec, C.c_void_p,
                                          MgpuVec, MgpuCol, MgpuCol, C.c_void_p]),
    'mgpu_parallel_transport': (C.c_int, [C.c_int64, MgpuVec, MgpuVec, MgpuVec, MgpuVec,
                                          C.c_void_p]),
    'mgpu_generate_photons': (C.c_int, [C.POINTER(MgpuSource), MgpuVec, MgpuVec, MgpuVec, MgpuCol,
                                        MgpuCol, C.c_void_p]),
    'mgpu_pose_adjoint': (C.c_int, [C.POINTER(MgpuAdjointProblem), C.c_void_p, C.c_int32,
                                    C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
    'mgpu_order_stats_workspace': (C.c_int64, [C.c_int64, C.c_int32]),
    'mgpu_order_stats': (C.c_int, [C.POINTER(MgpuStatsProblem), C.c_void_p]),
    'mgpu_facet_poses': (C.c_int, [C.POINTER(MgpuPoseUpdate), C.c_void_p]),
    'mgpu_fma_probe': (C.c_int, [C.c_int32, C.c_int32, C.c_int32, C.c_void_p, C.c_void_p]),
    'mgpu_philox4x32_10': (C.c_int, [C.c_void_p, C.c_void_p, C.c_int64, C.c_void_p]),
}

_lib = None


class LibraryNotBuilt(RuntimeError):
    pass


def load(path=LIB_PATH):
    """Load the CUDA library (once) and bind every entry point's signature."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise LibraryNotBuilt('%s is missing: build it with `python -c "import __graft_entry__ as g; '
                              'g.build()"` (there is no CPU fallback)' % path)
    lib = C.CDLL(path)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    if lib.mgpu_abi_version() != MGPU_ABI_VERSION:
        raise RuntimeError('libmarxs_gb300 ABI version mismatch')
    _lib = lib
    return lib


def check(code, what):
    if code != 0:
        raise RuntimeError('%s failed with CUDA error %d' % (what, code))


def col(t, stride=1):
    """MgpuCol for a device tensor (or None -> absent column)."""
    if t is None:
        return MgpuCol(None, 0)
    return MgpuCol(t.data_ptr(), stride)


def vec_aos(t):
    """MgpuVec over an (N, 4) row-major tensor (homogeneous coordinates)."""
    return MgpuVec(t.data_ptr(), t.stride(0), t.stride(1))


def vec_soa(t):
    """MgpuVec over a (3, N) tensor of component planes."""
    return MgpuVec(t.data_ptr(), t.stride(1), t.stride(0))
