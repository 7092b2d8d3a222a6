"""ctypes binding of libwhalegpu.so (the C ABI declared in include/whalegpu.h).

The library is built in-tree by ``build.py``.  There is no fallback: if the
shared object is missing or fails to load, every call that needs it raises.
With WG_HOST_LIBRARY=1 in the environment the host parts alone are loaded
(libwhalehost.so: model, ALE reader, packer, workload generator, tracking);
the device entry points are then absent and calling one raises.
"""
from __future__ import annotations

import ctypes as C
import os

from . import build as _build

WG_OK = 0
WG_EINVAL, WG_EPARSE, WG_ECUDA, WG_ENOMEM, WG_ESTATE, WG_ERANGE = -1, -2, -3, -4, -5, -6
NODE_LEAF, NODE_INTERNAL, NODE_WGD, NODE_ROOT = 0, 1, 2, 3
COND_NONE, COND_ROOT, COND_NONEXTINCT, COND_NOWHERE = 0, 1, 2, 3
BATCH_GRAD, BATCH_TABLES, BATCH_SCRATCH_ROWS, BATCH_CHECKPOINT, BATCH_PERSISTENT = 1, 2, 4, 8, 16
SYNTH_WALK, SYNTH_PUSH = 1, 2

_ERRNAMES = {WG_EINVAL: "EINVAL", WG_EPARSE: "EPARSE", WG_ECUDA: "ECUDA", WG_ENOMEM: "ENOMEM",
             WG_ESTATE: "ESTATE", WG_ERANGE: "ERANGE"}


class WhaleError(RuntimeError):
    """A libwhalegpu call returned a non-zero status."""

    def __init__(self, code: int, msg: str):
        super().__init__(f"[{_ERRNAMES.get(code, code)}] {msg}")
        self.code = code


_lib = None

vp = C.c_void_p
i32 = C.c_int32
i64 = C.c_int64
u32 = C.c_uint32
u64 = C.c_uint64
dbl = C.c_double
P_i32 = C.POINTER(C.c_int32)
P_i64 = C.POINTER(C.c_int64)
P_dbl = C.POINTER(C.c_double)
P_vp = C.POINTER(C.c_void_p)


def _declare(L):
    sigs = {
        "wg_last_error": (C.c_char_p, []),
        "wg_version": (C.c_int, []),
        "wg_ctx_create": (C.c_int, [C.c_int, P_vp]),
        "wg_ctx_destroy": (C.c_int, [vp]),
        "wg_ctx_stream": (vp, [vp]),
        "wg_ctx_set_timing": (C.c_int, [vp, C.c_int]),
        "wg_ctx_timings": (C.c_int, [vp, C.POINTER(C.c_float), C.POINTER(C.c_float), C.POINTER(C.c_float)]),
        "wg_probe_fp64": (C.c_int, [vp, P_dbl]),
        "wg_model_create": (C.c_int, [i32, P_i32, P_i32, P_i32, P_i32, P_dbl, P_dbl, P_i32, P_i32, i32, P_vp]),
        "wg_model_destroy": (C.c_int, [vp]),
        "wg_model_set_rates": (C.c_int, [vp, P_dbl, P_dbl, P_dbl, dbl, P_dbl]),
        "wg_model_set_tables": (C.c_int, [vp, P_dbl, P_dbl, P_dbl, P_dbl, dbl]),
        "wg_model_get_tables": (C.c_int, [vp, P_dbl, P_dbl, P_dbl]),
        "wg_model_condition": (C.c_int, [vp, P_dbl]),
        "wg_ccd_parse_ale": (C.c_int, [C.c_char_p, C.c_size_t, C.POINTER(C.c_char_p), P_i32, i32, P_vp]),
        "wg_ccd_read_ale_files": (C.c_int, [C.POINTER(C.c_char_p), i32, C.POINTER(C.c_char_p), P_i32, i32, i32, P_vp,
                                            P_i32]),
        "wg_ccd_create": (C.c_int, [i32, P_i32, P_i32, P_i32, P_i32, P_i32, P_i32, P_dbl, i64, P_vp]),
        "wg_ccd_destroy": (C.c_int, [vp]),
        "wg_ccd_info": (C.c_int, [vp, P_i32, P_i32, P_i64, P_i32]),
        "wg_ccd_export": (C.c_int, [vp, P_i32, P_i64, P_i32, P_i32, P_i32, P_i32, P_i32, P_dbl]),
        "wg_batch_create": (C.c_int, [vp, vp, P_vp, i32, u32, P_vp]),
        "wg_batch_destroy": (C.c_int, [vp]),
        "wg_pack_info": (C.c_int, [vp, P_vp, i32, u32, P_i64, P_i64, P_i64, P_i64, P_dbl]),
        "wg_pack_tasks": (C.c_int, [vp, P_vp, i32, u32, P_i32, i64, P_i64]),
        "wg_batch_info": (C.c_int, [vp, P_i32, P_i32, P_i64, P_dbl, P_dbl, P_dbl]),
        "wg_batch_launches": (C.c_int, [vp, P_i32, P_i32]),
        "wg_batch_tables_layout": (C.c_int, [vp, P_i32, P_i32, P_i64, P_i64]),
        "wg_nowhere_condition": (C.c_int, [vp, vp, P_dbl, P_dbl, P_dbl, P_dbl, P_dbl]),
        "wg_backtrack": (C.c_int, [vp, vp, vp, C.c_int32, C.c_int32, C.c_uint64, C.c_char_p, C.c_int64, P_i64]),
        "wg_backtrack_tables": (C.c_int, [vp, vp, P_dbl, C.c_int64, C.c_int32, C.c_uint64, C.c_char_p, C.c_int64,
                                          P_i64]),
        "wg_logpdf": (C.c_int, [vp, vp, vp, P_dbl, P_dbl]),
        "wg_logpdf_grad": (C.c_int, [vp, vp, vp, P_dbl, P_dbl, P_dbl, P_dbl, P_dbl, P_dbl, P_dbl, P_dbl, P_dbl]),
        "wg_logpdf_grad_weighted": (C.c_int, [vp, vp, vp, P_dbl, C.c_double, P_dbl, P_dbl, P_dbl, P_dbl, P_dbl, P_dbl,
                                              P_dbl, P_dbl, P_dbl]),
        "wg_logpdf_plain": (C.c_int, [vp, vp, vp, P_dbl, P_dbl]),
        "wg_logpdf_noalloc": (C.c_int, [vp, vp, vp, P_dbl, P_dbl]),
        "wg_logpdf_tables": (C.c_int, [vp, vp, vp, i32, P_dbl, i64, P_i64, P_dbl]),
        "wg_batch_tables": (C.c_int, [vp, vp, i32, P_dbl, i64, P_i64, P_dbl]),
        "wg_track_device": (C.c_int, [vp, vp, vp, i32, P_i32, C.POINTER(C.c_uint64), P_i64]),
        "wg_track_nodes": (C.c_int, [vp, P_i32, i64]),
        "wg_tree_newick": (C.c_int, [vp, vp, P_i32, i32, C.c_char_p, i64, P_i64]),
        "wg_enqueue": (C.c_int, [vp, vp, vp, C.c_int]),
        "wg_fetch": (C.c_int, [vp, vp, vp, P_dbl, P_dbl, P_dbl, P_dbl, P_dbl, P_dbl]),
        "wg_synth_family": (C.c_int, [vp, P_dbl, P_dbl, P_dbl, dbl, C.POINTER(C.c_char_p), u64, i32, i32, i32, i32,
                                      i32, C.c_char_p, i64, P_i64]),
    }
    host_only = os.path.basename(getattr(L, "_name", "") or "") == os.path.basename(_build.HOST_LIB)
    for name, (res, args) in sigs.items():
        if host_only and not hasattr(L, name):
            continue  # a device entry point: absent from the host library
        f = getattr(L, name)
        f.restype = res
        f.argtypes = args
    return L


def lib():
    """Load (building first if needed) libwhalegpu.so; raises if it cannot."""
    global _lib
    if _lib is None:
        host_only = os.environ.get("WG_HOST_LIBRARY") == "1"
        path = _build.HOST_LIB if host_only else _build.LIB
        if not os.path.exists(path):
            _build.build()
        _lib = _declare(C.CDLL(path))
    return _lib


def check(status: int) -> None:
    if status != WG_OK:
        msg = lib().wg_last_error().decode(errors="replace")
        raise WhaleError(status, msg)


def dptr(a):
    return a.ctypes.data_as(P_dbl) if a is not None else None


def iptr(a):
    return a.ctypes.data_as(P_i32) if a is not None else None


def lptr(a):
    return a.ctypes.data_as(P_i64) if a is not None else None
