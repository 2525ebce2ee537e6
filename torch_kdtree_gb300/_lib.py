"""ctypes binding of libtkknn.so (the C ABI declared in include/tk_knn.h).

The library is the only implementation of every query path: if it is missing
or cannot be loaded, importing this module raises -- there is no fallback.
"""
from __future__ import annotations

import ctypes
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libtkknn.so")

TK_OK = 0
TK_HOST_AUTO, TK_HOST_DIRECT, TK_HOST_STAGED = 0, 1, 2  # tk_tree_query_host transfers
TK_EINVAL = 1
TK_ENOMEM = 2
TK_EUNSUPPORTED = 3
TK_ETIMEOUT = 4
TK_ECUDA = 5
TK_EWORKSPACE = 6
TK_F32 = 0
TK_F64 = 1
TK_BRUTE_EXACT = 0
TK_BRUTE_TF32 = 1
TK_BRUTE_BF16_SPLIT = 2
TK_NOALLOC_MAX_QUERIES = 262144

_STATUS_NAMES = {
    TK_EINVAL: "EINVAL", TK_ENOMEM: "ENOMEM", TK_EUNSUPPORTED: "EUNSUPPORTED",
    TK_ETIMEOUT: "ETIMEOUT", TK_ECUDA: "ECUDA", TK_EWORKSPACE: "EWORKSPACE",
}


class TkError(RuntimeError):
    """A tk_* entry point returned a non-zero status."""

    def __init__(self, status: int, msg: str):
        super().__init__(f"{msg} [{_STATUS_NAMES.get(status, status)}]")
        self.status = status


class TreeInfo(ctypes.Structure):
    _fields_ = [("n_points", ctypes.c_int64), ("dims", ctypes.c_int32), ("dtype", ctypes.c_int32),
                ("levels", ctypes.c_int32), ("device", ctypes.c_int32), ("n_leaves", ctypes.c_int64),
                ("device_bytes", ctypes.c_int64)]


class QueryOpts(ctypes.Structure):
    _fields_ = [("threads_per_query", ctypes.c_int32), ("bin_queries", ctypes.c_int32),
                ("smem_levels", ctypes.c_int32), ("block_threads", ctypes.c_int32),
                ("blocks_per_sm", ctypes.c_int32), ("kernel_start_event", ctypes.c_void_p),
                ("kernel_stop_event", ctypes.c_void_p), ("prune_boxes", ctypes.c_int32),
                ("traversal", ctypes.c_int32)]

    @classmethod
    def make(cls, threads_per_query=0, bin_queries=-1, smem_levels=-1, block_threads=0, blocks_per_sm=0,
             kernel_start_event=None, kernel_stop_event=None, prune_boxes=-1, traversal=0):
        return cls(threads_per_query, bin_queries, smem_levels, block_threads, blocks_per_sm,
                   kernel_start_event, kernel_stop_event, prune_boxes, traversal)


_vp = ctypes.c_void_p
_i32 = ctypes.c_int32
_i64 = ctypes.c_int64
_int = ctypes.c_int
_sz = ctypes.c_size_t

# name -> (restype, argtypes)
SIGNATURES = {
    "tk_last_error": (ctypes.c_char_p, []),
    "tk_version": (_int, []),
    "tk_cuda_available": (_int, []),
    "tk_tree_create": (_int, [_vp, _i64, _int, _int, _int, _int, _int, ctypes.POINTER(_vp)]),
    "tk_tree_create_device": (_int, [_vp, _i64, _int, _int, _int, _int, _vp, ctypes.POINTER(_vp)]),
    "tk_tree_create_from_layout": (_int, [_vp, _vp, _vp, _vp, _i64, _int, _int, _int, _int, ctypes.POINTER(_vp)]),
    "tk_tree_destroy": (_int, [_vp]),
    "tk_tree_get_info": (_int, [_vp, ctypes.POINTER(TreeInfo)]),
    "tk_tree_get_perm": (_int, [_vp, _vp]),
    "tk_tree_get_points": (_int, [_vp, _vp]),
    "tk_tree_get_splits": (_int, [_vp, _vp, _vp]),
    "tk_tree_query_workspace_size": (_sz, [_vp, _i64]),
    "tk_tree_query": (_int, [_vp, _vp, _i64, _int, _vp, _vp, ctypes.POINTER(QueryOpts), _vp, _sz, _vp]),
    "tk_batch_create": (_int, [ctypes.POINTER(_vp), _int, ctypes.POINTER(_i64), ctypes.POINTER(_i32),
                                ctypes.POINTER(_vp)]),
    "tk_batch_destroy": (_int, [_vp]),
    "tk_batch_workspace_size": (_sz, [_vp]),
    "tk_batch_output_size": (_i64, [_vp]),
    "tk_batch_query": (_int, [_vp, _vp, _vp, _vp, _int, _int, _vp, _sz, _vp]),
    "tk_nn_distance_workspace_size": (_sz, [_i64, _i64, _int, _int, _int, _int]),
    "tk_nn_distance": (_int, [_vp, _i64, _vp, _i64, _int, _int, _int, _int, _vp, _vp, _vp, _sz, _vp]),
    "tk_tree_query_noalloc": (_int, [_vp, _vp, _i64, _int, _vp, _vp, ctypes.POINTER(QueryOpts), _vp]),
    "tk_tree_query_host": (_int, [_vp, _vp, _i64, _int, _vp, _vp, ctypes.POINTER(QueryOpts), _int, _vp]),
    "tk_tree_query_cpu": (_int, [_vp, _vp, _i64, _int, _vp, _vp, _int]),
    "tk_nn_distance_report": (_int, [_vp, _i64, _i64, _int, _int, _int, _int, ctypes.POINTER(_int),
                                     ctypes.POINTER(_int)]),
    "tk_set_device_wait_limit": (ctypes.c_uint32, [ctypes.c_uint32]),
    "tk_knn_backward_workspace_size": (_sz, [_i64, _int, _i64]),
    "tk_knn_backward": (_int, [_vp, _vp, _vp, _vp, _i64, _i64, _int, _int, _int, _vp, _vp, _vp, _sz, _vp]),
}


def _load():
    if not os.path.exists(LIB_PATH):
        raise ImportError(
            f"{LIB_PATH} is not built. Build it with `python -c \"import __graft_entry__ as g; g.build()\"` "
            "(needs nvcc); this package has no non-CUDA implementation.")
    lib = ctypes.CDLL(LIB_PATH)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    return lib


LIB = _load()


def last_error() -> str:
    return LIB.tk_last_error().decode(errors="replace")


def check(status: int) -> None:
    if status != TK_OK:
        raise TkError(status, last_error())
