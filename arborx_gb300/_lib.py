"""ctypes binding of libarborx_gb300.so (the C ABI of include/arborx_gb300.h).

Loading fails loudly when the library has not been built: there is no CPU
fallback anywhere in this package.
"""

import ctypes
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libarborx_gb300.so")

# abx_status
SUCCESS = 0
ERROR_INVALID_ARGUMENT = 1
ERROR_CUDA = 2
ERROR_OUT_OF_MEMORY = 3
ERROR_BUFFER_OVERFLOW = 4
ERROR_DEVICE = 5
ERROR_NOT_SUPPORTED = 6
ERROR_TIMEOUT = 7

# abx_geometry
POINT, BOX, SPHERE, RAY = 0, 1, 2, 3
# KDOP<3, k> geometry kinds and their number of directions (k / 2)
KDOP6, KDOP14, KDOP18, KDOP26 = 4, 5, 6, 7
KDOP_NDIR = {KDOP6: 3, KDOP14: 7, KDOP18: 9, KDOP26: 13}

# Every function the header declares: name -> (restype, argtypes)
_P = ctypes.c_void_p
_I64 = ctypes.c_int64
_I32 = ctypes.c_int32
_STATUS = ctypes.c_int


class DeviceViewC(ctypes.Structure):
    _fields_ = [("nodes", ctypes.c_void_p), ("leaves", ctypes.c_void_p), ("size", ctypes.c_int64),
                ("geometry", ctypes.c_int32), ("reserved", ctypes.c_int32)]


class TraversalPolicyC(ctypes.Structure):
    _fields_ = [("buffer_size", ctypes.c_int32), ("sort_predicates", ctypes.c_int32)]


class ServerConfigC(ctypes.Structure):
    _fields_ = [("workers", ctypes.c_int32), ("l2_persist", ctypes.c_int32),
                ("max_inflight_bytes", ctypes.c_int64), ("max_batch_queries", ctypes.c_int64)]


class RequestC(ctypes.Structure):
    _fields_ = [("tree", ctypes.c_int32), ("kind", ctypes.c_int32), ("h_queries", ctypes.c_void_p),
                ("nq", ctypes.c_int64), ("k", ctypes.c_int32), ("reserved", ctypes.c_int32)]


class ServerStatisticsC(ctypes.Structure):
    _fields_ = [("completed_requests", ctypes.c_int64), ("completed_queries", ctypes.c_int64),
                ("batches", ctypes.c_int64), ("p50_ms", ctypes.c_double), ("p99_ms", ctypes.c_double),
                ("span_s", ctypes.c_double)]


REQ_NEAREST = 0
REQ_INTERSECTS = 1

class ValuesC(ctypes.Structure):
    _fields_ = [("data", ctypes.c_void_p), ("value_stride", ctypes.c_int64),
                ("coord_stride", ctypes.c_int64)]


SIGNATURES = {
    "abx_status_string": (ctypes.c_char_p, [_STATUS]),
    "abx_last_error": (ctypes.c_char_p, []),
    "abx_version": (ctypes.c_char_p, []),
    "abx_device_errors": (_STATUS, [_P, ctypes.POINTER(ctypes.c_uint32)]),
    "abx_tuning_set": (_STATUS, [ctypes.c_char_p, _I32]),
    "abx_tuning_reset": (_STATUS, []),
    "abx_profiling_enable": (_STATUS, [_I32]),
    "abx_profiling_stage": (_STATUS, [ctypes.c_char_p, ctypes.POINTER(ctypes.c_double), ctypes.POINTER(_I64)]),
    "abx_profiling_reset": (_STATUS, []),
    "abx_bvh_create": (_STATUS, [_P, ctypes.c_int, _P, _I64, ctypes.POINTER(_P)]),
    "abx_bvh_create_strided": (_STATUS, [_P, ctypes.c_int, ValuesC, _I64, ctypes.POINTER(_P)]),
    "abx_gather_rows": (_STATUS, [_P, _P, _I64, _I64, _P, _I64, _P]),
    "abx_kdop_from_geometry": (_STATUS, [_P, ctypes.c_int, _P, _I64, ctypes.c_int, _P]),
    "abx_bvh_kdop_bounds": (_STATUS, [_P, _P]),
    "abx_bvh_save": (_STATUS, [_P, ctypes.c_char_p]),
    "abx_bvh_load": (_STATUS, [_P, ctypes.c_char_p, ctypes.POINTER(_P)]),
    "abx_bvh_destroy": (_STATUS, [_P]),
    "abx_bvh_size": (_I64, [_P]),
    "abx_bvh_bounds": (_STATUS, [_P, _P]),
    "abx_bvh_geometry": (ctypes.c_int, [_P]),
    "abx_bvh_export_nodes": (_STATUS, [_P, _P, _P, _P]),
    "abx_bvh_device_view": (_STATUS, [_P, ctypes.POINTER(DeviceViewC)]),
    "abx_bvh_query_intersects": (
        _STATUS,
        [_P, _P, ctypes.c_int, _P, _I64, TraversalPolicyC, ctypes.POINTER(_P)],
    ),
    "abx_bvh_query_nearest": (
        _STATUS,
        [_P, _P, _P, _I64, _P, _I32, TraversalPolicyC, _I32, ctypes.POINTER(_P)],
    ),
    "abx_forest_create": (_STATUS, [_P, ctypes.c_int, _P, _P, _I32, ctypes.POINTER(_P)]),
    "abx_forest_destroy": (_STATUS, [_P]),
    "abx_forest_num_trees": (_I32, [_P]),
    "abx_forest_size": (_I64, [_P, _I32]),
    "abx_forest_bounds": (_STATUS, [_P, _I32, _P]),
    "abx_forest_export_nodes": (_STATUS, [_P, _I32, _P, _P, _P]),
    "abx_forest_query_intersects": (
        _STATUS,
        [_P, _P, ctypes.c_int, _P, _P, TraversalPolicyC, ctypes.POINTER(_P)],
    ),
    "abx_forest_query_nearest": (
        _STATUS,
        [_P, _P, _P, _P, _P, _I32, TraversalPolicyC, _I32, ctypes.POINTER(_P)],
    ),
    "abx_brute_create": (_STATUS, [_P, ctypes.c_int, _P, _I64, ctypes.POINTER(_P)]),
    "abx_brute_destroy": (_STATUS, [_P]),
    "abx_brute_size": (_I64, [_P]),
    "abx_brute_bounds": (_STATUS, [_P, _P]),
    "abx_brute_query_intersects": (
        _STATUS,
        [_P, _P, ctypes.c_int, _P, _I64, TraversalPolicyC, ctypes.POINTER(_P)],
    ),
    "abx_brute_query_nearest": (
        _STATUS,
        [_P, _P, _P, _I64, _P, _I32, TraversalPolicyC, _I32, ctypes.POINTER(_P)],
    ),
    "abx_server_create": (_STATUS, [ctypes.POINTER(ServerConfigC), ctypes.POINTER(_P)]),
    "abx_server_destroy": (_STATUS, [_P]),
    "abx_server_add_tree": (_STATUS, [_P, _P, ctypes.POINTER(_I32)]),
    "abx_server_submit": (_STATUS, [_P, ctypes.POINTER(RequestC), ctypes.POINTER(_I64)]),
    "abx_server_wait": (_STATUS, [_P, _I64, ctypes.POINTER(_I64), ctypes.POINTER(ctypes.c_double)]),
    "abx_server_result": (_STATUS, [_P, _I64, _P, _P, _P]),
    "abx_server_stats": (_STATUS, [_P, ctypes.POINTER(ServerStatisticsC)]),
    "abx_server_reset_stats": (_STATUS, [_P]),
    "abx_bvh_query_ordered_intersects": (
        _STATUS, [_P, _P, _P, _I64, _I32, TraversalPolicyC, _I32, ctypes.POINTER(_P)],
    ),
    "abx_bvh_query_nearest_host": (_STATUS, [_P, _P, _P, _I64, ctypes.c_int32, TraversalPolicyC, _I64,
                                             _P, _P, _P]),
    "abx_bvh_query_nearest_into": (
        _STATUS, [_P, _P, _P, _I64, _I32, TraversalPolicyC, _P, _P, _P],
    ),
    "abx_find_neighbor_list": (_STATUS, [_P, _P, _I64, ctypes.c_float, _I32, ctypes.POINTER(_P)]),
    "abx_expand_half_to_full": (_STATUS, [_P, _I64, _P, _P, ctypes.POINTER(_P)]),
    "abx_crs_num_queries": (_I64, [_P]),
    "abx_crs_num_results": (_I64, [_P]),
    "abx_crs_offsets": (_P, [_P]),
    "abx_crs_indices": (_P, [_P]),
    "abx_crs_distances": (_P, [_P]),
    "abx_crs_destroy": (_STATUS, [_P]),
    "abx_scene_bounds": (_STATUS, [_P, ctypes.c_int, _P, _I64, _P]),
    "abx_morton64": (_STATUS, [_P, ctypes.c_int, _P, _I64, _P, _P]),
    "abx_morton32": (_STATUS, [_P, ctypes.c_int, _P, _I64, _P, _P]),
    "abx_sort_u64": (_STATUS, [_P, _P, _I64, _P]),
    "abx_sort_u32": (_STATUS, [_P, _P, _I64, _P]),
    "abx_generate_hierarchy": (_STATUS, [_P, ctypes.c_int, _P, _I64, _P, _P, _P, _P]),
    "abx_exclusive_scan_i32": (_STATUS, [_P, _P, _I64, _P]),
    "abx_exclusive_scan_i32_noalloc": (_STATUS, [_P, _P, _I64, _P]),
}

# Largest input of abx_exclusive_scan_i32_noalloc (ABX_NOALLOC_SCAN_MAX_N).
NOALLOC_SCAN_MAX_N = 16777216


class AbxError(RuntimeError):
    """A failing call of the C ABI (status + the library's message)."""

    def __init__(self, status, message):
        super().__init__(message)
        self.status = status


class SearchException(AbxError):
    """Mirror of ArborX::SearchException (src/misc/ArborX_Exception.hpp:19-37),
    raised for ABX_ERROR_BUFFER_OVERFLOW and invalid arguments."""


_lib = None


def load(path=LIB_PATH):
    """Load the shared library; raises ImportError if it is missing."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise ImportError(
            "libarborx_gb300.so is not built (expected at %s); run "
            "`python -c 'import arborx_gb300.build as b; b.build()'`" % path
        )
    L = ctypes.CDLL(path)
    for name, (res, args) in SIGNATURES.items():
        f = getattr(L, name)
        f.restype = res
        f.argtypes = args
    _lib = L
    return L


def check(status):
    if status == SUCCESS:
        return
    L = load()
    name = L.abx_status_string(status).decode()
    msg = "%s: %s" % (name, L.abx_last_error().decode())
    if status in (ERROR_BUFFER_OVERFLOW, ERROR_INVALID_ARGUMENT):
        raise SearchException(status, msg)
    raise AbxError(status, msg)
