"""ctypes binding of libvissat_gb300.so (the C ABI declared in include/vissat_gb300.h).

The shared library is the product: there is no CPU fallback.  Loading fails loudly if
the library has not been built (``python -m vissatsatellitestereo_gb300.build``), and
every call raises ``VsError`` with the library's message on a non-zero status.
"""
import ctypes
import os

import numpy as np

LIB_PATH = os.path.join(os.path.dirname(os.path.abspath(__file__)), 'libvissat_gb300.so')

VS_OK = 0
VS_ERR_ARG = 1
VS_ERR_CUDA = 2
VS_ERR_WORKSPACE = 3
VS_ERR_FACTORIZE = 4
VS_ERR_DEGENERATE = 5
VS_ERR_TIMEOUT = 6

VS_PROJ_EXACT = 0
VS_PROJ_FAST = 1
VS_LAYOUT_HWV = 0
VS_LAYOUT_VHW = 1
VS_CAMERA_PARAMS = 14
VS_ERROR_STATS = 6
VS_FUSE_STATIC_MAX_CELLS = 4194304
VS_CUBE_FP32 = 0
VS_CUBE_BF16X3 = 1
VS_CUBE_TF32X3 = 2
VS_CUBE_BF16X6 = 3
VS_CUBE_BF16X3_TC = 4
VS_CUBE_BF16X3_LIN = 5
VS_CUBE_BF16X3_LIN_TC = 6
VS_CUBE_MAX_CAMERAS = 128
VS_GEO_EXACT = 0
VS_GEO_FAST = 1
VS_GEO_FAST_TOL_M = 2.5e-7
VS_GEO_FLAG_HEMISPHERE = 1

# VsRpcCamera: 92 doubles in declaration order
CAMERA_DOUBLES = 92

_vp = ctypes.c_void_p
_i64 = ctypes.c_int64
_int = ctypes.c_int
_dbl = ctypes.c_double
_sz = ctypes.c_size_t

# name -> (restype, argtypes)
SIGNATURES = {
    'vs_version': (ctypes.c_char_p, []),
    'vs_last_error': (ctypes.c_char_p, []),
    'vs_rpc_project': (_int, [_vp, _int, _vp, _vp, _vp, _i64, _i64, _vp, _vp, _vp, _int, _vp]),
    'vs_rpc_project_cube_workspace_size': (_sz, [_int]),
    'vs_rpc_project_cube': (_int, [_vp, _int, _vp, _i64, _vp, _int, _vp, _sz, _vp]),
    'vs_rpc_project_cube_status': (_int, [_vp, _int, _int, _vp]),
    'vs_map_points': (_int, [_vp, _i64, _int, _int, _i64, _i64, _i64, _i64, _i64, _i64, _vp, _vp]),
    'vs_map_upload': (_int, [_vp, _i64, _int, _int, _vp, _i64, _vp]),
    'vs_set_tc_wait_limit': (None, [ctypes.c_uint]),
    'vs_set_binning_ctas_per_sm': (None, [ctypes.c_int]),
    'vs_set_l2_persisting': (_int, [_sz]),
    'vs_rpc_inverse_project_workspace_size': (_sz, [_int, _i64]),
    'vs_rpc_inverse_project': (_int, [_vp, _int, _vp, _vp, _vp, _i64, _i64, _int, _vp, _vp, _vp, _int, _vp, _vp, _sz,
                                      _vp]),
    'vs_affine_fit_workspace_size': (_sz, [_int, _i64]),
    'vs_affine_fit': (_int, [_vp, _vp, _vp, _i64, _vp, _vp, _vp, _int, _i64, _vp, _vp, _vp, _sz, _vp]),
    'vs_camera_approx_affine_workspace_size': (_sz, [_int, _i64]),
    'vs_camera_approx_affine': (_int, [_vp, _int, _vp, _vp, _vp, _i64, _i64, _vp, _vp, _vp, _sz, _vp]),
    'vs_dlt_fit_workspace_size': (_sz, [_int, _i64]),
    'vs_dlt_fit': (_int, [_vp, _vp, _vp, _i64, _vp, _vp, _vp, _int, _i64, _vp, _vp, _vp, _vp, _vp, _sz, _vp]),
    'vs_perspective_error_workspace_size': (_sz, [_int, _i64]),
    'vs_perspective_error': (_int, [_vp, _vp, _vp, _i64, _vp, _vp, _vp, _int, _i64, _vp, _vp, _vp, _vp, _vp,
                                    _sz, _vp]),
    'vs_camera_approx_workspace_size': (_sz, [_int, _i64]),
    'vs_camera_approx_perspective': (_int, [_vp, _int, _vp, _vp, _vp, _vp, _vp, _vp, _i64, _i64, _int, _vp,
                                            _vp, _vp, _vp, _sz, _vp]),
    'vs_proj_to_grid_workspace_size': (_sz, [_i64, _i64]),
    'vs_proj_to_grid': (_int, [_vp, _i64, _dbl, _dbl, _dbl, _dbl, _i64, _i64, _vp, _vp, _sz, _vp]),
    'vs_median_blur3x3_f32': (_int, [_vp, _vp, _i64, _i64, _i64, _vp]),
    'vs_median_blur3x3_f64': (_int, [_vp, _vp, _i64, _i64, _i64, _vp]),
    'vs_dsm_from_points_workspace_size': (_sz, [_int, _i64, _i64]),
    'vs_dsm_from_points': (_int, [_vp, _vp, _int, _dbl, _dbl, _dbl, _dbl, _i64, _i64, _vp, _vp, _sz, _vp]),
    'vs_aoi_batch_plan_workspace_size': (_sz, [_vp, _int, _int]),
    'vs_aoi_batch_plan': (_int, [_vp, _int, _vp, _int, _int, _vp, _sz, _vp, _vp]),
    'vs_aoi_batch_query': (_int, [_vp, _vp, _vp, _vp]),
    'vs_aoi_batch_run': (_int, [_vp, _int, _int, _int, _vp, _vp]),
    'vs_aoi_batch_fuse': (_int, [_vp, _int, _int, _vp, _vp, _int, _vp, _sz, _vp]),
    'vs_aoi_batch_destroy': (None, [_vp]),
    'vs_dsm_from_points_overlap_workspace_size': (_sz, [_int, _i64, _i64]),
    'vs_dsm_from_points_overlap': (_int, [_vp, _vp, _int, _dbl, _dbl, _dbl, _dbl, _i64, _i64, _vp, _vp, _sz, _vp, _vp,
                                          _vp]),
    'vs_dsm_from_points_pipelined_workspace_size': (_sz, [_int, _i64, _i64]),
    'vs_dsm_from_points_pipelined': (_int, [_vp, _vp, _int, _dbl, _dbl, _dbl, _dbl, _i64, _i64, _vp, _vp, _sz,
                                            _vp, _vp]),
    'vs_fuse_dsms_workspace_size': (_sz, [_i64, _i64]),
    'vs_fuse_dsms': (_int, [_vp, _int, _i64, _i64, _i64, _vp, _int, _vp, _sz, _vp]),
    'vs_fuse_dsms_static': (_int, [_vp, _int, _i64, _i64, _i64, _vp, _int, _vp]),
    'vs_dsm_from_points_host_workspace_size': (_sz, [_i64, _int, _i64, _i64]),
    'vs_dsm_from_points_host': (_int, [_vp, _vp, _int, _dbl, _dbl, _dbl, _dbl, _i64, _i64, _vp, _int, _vp, _sz, _vp,
                                       _vp]),
    'vs_geo_plan_device_bytes': (_sz, []),
    'vs_geo_plan_create': (_int, [_vp, _vp, _sz, _vp, _vp]),
    'vs_geo_plan_query': (_int, [_vp, _vp, _vp]),
    'vs_geo_plan_destroy': (None, [_vp]),
    'vs_enu_to_geodetic': (_int, [_vp, _vp, _i64, _i64, _vp, _vp, _vp, _vp]),
    'vs_geodetic_to_utm': (_int, [_vp, _vp, _vp, _i64, _vp, _vp, _vp, _vp]),
    'vs_depth_to_points_workspace_size': (_sz, [_i64, _i64]),
    'vs_depth_to_points': (_int, [_vp, _i64, _i64, _vp, _vp, _int, _vp, _vp, _vp, _vp, _sz, _vp]),
    'vs_dsm_from_depth_maps_workspace_size': (_sz, [_i64, _i64]),
    'vs_dsm_from_depth_maps': (_int, [_vp, _vp, _vp, _int, _vp, _vp, _int, _dbl, _dbl, _dbl, _dbl, _i64, _i64, _vp,
                                      _vp, _vp, _sz, _vp]),
}


class VsGeoFrame(ctypes.Structure):
    _fields_ = [('lat0', _dbl), ('lon0', _dbl), ('alt0', _dbl), ('utm_zone', ctypes.c_int32),
                ('south', ctypes.c_int32), ('box_lo', _dbl * 3), ('box_hi', _dbl * 3)]


class VsError(RuntimeError):
    def __init__(self, status, message):
        super().__init__(f'vissat-gb300 status {status}: {message}')
        self.status = status


_lib = None


def lib():
    """The loaded library (loaded on first use)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError(f'{LIB_PATH} is missing: build it with '
                              '`python -m vissatsatellitestereo_gb300.build` (needs nvcc)')
        handle = ctypes.CDLL(LIB_PATH)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(handle, name)
            fn.restype = res
            fn.argtypes = args
        _lib = handle
    return _lib


def check(status):
    if status != VS_OK:
        raise VsError(status, lib().vs_last_error().decode())


def call(name, *args):
    check(getattr(lib(), name)(*args))


def camera_array(meta_dicts):
    """(C, 92) float64 rows in VsRpcCamera field order from reference meta_dicts."""
    rows = []
    for m in meta_dicts:
        r = m['rpc']
        row = [r['rowOff'], r['rowScale'], r['colOff'], r['colScale'], r['latOff'], r['latScale'],
               r['lonOff'], r['lonScale'], r['altOff'], r['altScale']]
        for key in ('rowNum', 'rowDen', 'colNum', 'colDen'):
            coeffs = [float(c) for c in r[key]]
            if len(coeffs) != 20:
                raise ValueError(f'{key} must hold 20 coefficients, got {len(coeffs)}')
            row += coeffs
        row += [float(m['width']), float(m['height'])]
        rows.append(row)
    arr = np.asarray(rows, dtype=np.float64).reshape(-1, CAMERA_DOUBLES)
    return np.ascontiguousarray(arr)
