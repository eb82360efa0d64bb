"""ctypes binding of libgrafttn.so (the C ABI declared in include/grafttn.h).

The shared library is built in-tree next to this package (``graft.jl_gb300/libgrafttn.so``).
There is no fallback: importing the device layer without the library raises ImportError.
"""
from __future__ import annotations

import ctypes as C
import os

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(os.path.dirname(_HERE), "libgrafttn.so")

GTN_OK = 0
GTN_ERR_INVALID = 1
GTN_ERR_SHAPE = 2
GTN_ERR_MEMORY = 3
GTN_ERR_CUDA = 4
GTN_ERR_TIMEOUT = 5
GTN_ERR_UNSUPPORTED = 6
GTN_ERR_NOT_CONVERGED = 7

PREC_FP64 = 0
PREC_BF16X6 = 1
PREC_BF16X3 = 2
PREC_FP32 = 3
PREC_FP16X3 = 4
PREC_FP64E = 5
KERNEL_NAMES = {0: "small_contract", 1: "gather", 2: "split_bf16", 3: "zgemm_simt", 4: "cgemm_simt",
                5: "tc_gemm", 6: "convert", 7: "output_permute"}
PRECISIONS = {"fp64": PREC_FP64, "bf16x6": PREC_BF16X6, "bf16x3": PREC_BF16X3, "fp32": PREC_FP32,
              "fp16x3": PREC_FP16X3, "fp64e": PREC_FP64E}

# Every symbol declared in include/grafttn.h, with (restype, argtypes).
_p = C.c_void_p
_i = C.c_int
_i64 = C.c_int64
_d = C.c_double
_pi = C.POINTER(C.c_int)
_pi64 = C.POINTER(C.c_int64)
_pd = C.POINTER(C.c_double)
SIGNATURES = {
    "gtn_ctx_create": (_i, [_i, C.POINTER(_p)]),
    "gtn_ctx_destroy": (_i, [_p]),
    "gtn_ctx_set_stream": (_i, [_p, _p]),
    "gtn_ctx_stream": (_p, [_p]),
    "gtn_last_error": (C.c_char_p, [_p]),
    "gtn_ctx_launch_count": (_i64, [_p]),
    "gtn_ctx_sync": (_i, [_p]),
    "gtn_ctx_set_linalg_precision": (_i, [_p, _i]),
    "gtn_ctx_linalg_precision": (_i, [_p]),
    "gtn_map_create": (_i, [_p, _i, _pi, _pi64, _pi, _pi, _pi, C.POINTER(_p), _i, C.POINTER(_p)]),
    "gtn_map_destroy": (_i, [_p]),
    "gtn_map_apply": (_i, [_p, _p, _p]),
    "gtn_map_apply_prec": (_i, [_p, _i, _p, _p]),
    "gtn_map_apply_host": (_i, [_p, _p, _p]),
    "gtn_map_set_fp64": (_i, [_p, _p]),
    "gtn_map_apply_profiled": (_i, [_p, _i, _p, _p, _i, _pd, _pi, _pd, _pi]),
    "gtn_map_info": (_i, [_p, _pi64, _pi64, _pd, _pi, _pi64]),
    "gtn_map_apply_batched": (_i, [_i, C.POINTER(_p), C.POINTER(_p), C.POINTER(_p), _i]),
    "gtn_batch_create": (_i, [_i, C.POINTER(_p), C.POINTER(_p), C.POINTER(_p), _i, _i, C.POINTER(_p)]),
    "gtn_batch_run": (_i, [_p]),
    "gtn_batch_destroy": (_i, [_p]),
    "gtn_map_out_shape": (_i, [_p, _pi, _pi64]),
    "gtn_blockmap_create": (_i, [_p, _i, _pi, _pi, _p, _p, _i, _p, _i, C.POINTER(_p), _pi64, _pi64, _i, _d,
                                 C.POINTER(_p)]),
    "gtn_blockmap_apply": (_i, [_p, _p, _p]),
    "gtn_blockmap_set_graph": (_i, [_p, _i]),
    "gtn_blockmap_info": (_i, [_p, _pd, _pi, _pi64]),
    "gtn_blockmap_destroy": (_i, [_p]),
    "gtn_blockmap_lanczos_min": (_i, [_p, _p, _p, _i, _d, _i, _i, _pd, _pi, _pd]),
    "gtn_blockmap_lanczos_refine": (_i, [_p, _p, _p, _i, _d, _i, _pd, _pi, _pd]),
    "gtn_contract": (_i, [_p, _i, _pi, _pi64, _pi, _pi, _pi, C.POINTER(_p), _p, _i]),
    "gtn_contract_vjp": (_i, [_p, _i, _pi, _pi64, _pi, _pi, _pi, C.POINTER(_p), _i, _p, _p, _i]),
    "gtn_permute": (_i, [_p, _i, _pi64, _pi, _p, _p]),
    "gtn_lanczos_min": (_i, [_p, _p, _i, _d, _i, _i, _pd, _pi, _pd]),
    "gtn_lanczos_refine": (_i, [_p, _p, _i, _d, _i, _pd, _pi, _pd]),
    "gtn_expm_apply": (_i, [_p, _d, _d, _p, _i, _d, _pi]),
    "gtn_expm_apply_arnoldi": (_i, [_p, _d, _d, _p, _i, _d, _pi]),
    "gtn_expm_small": (_i, [_i, _pd, _pd]),
    "gtn_svd_trunc": (_i, [_p, _i64, _i64, _p, _i64, _d, _d, _d, _p, _pd, _p, _pi64, _pd]),
    "gtn_qr": (_i, [_p, _i64, _i64, _p, _p, _p]),
    "gtn_dot": (_i, [_p, _i64, _p, _p, _pd]),
    "gtn_axpby": (_i, [_p, _i64, _d, _d, _p, _d, _d, _p]),
    "gtn_diag_scale": (_i, [_p, _i64, _i64, _pd, _i, _p]),
    "gtn_copy2d": (_i, [_p, _i64, _i64, _p, _i64, _p, _i64]),
    "gtn_restrict_leg": (_i, [_p, _i, _pi64, _i, _i64, _pi64, _p, _p]),
    "gtn_fill": (_i, [_p, _i64, _d, _d, _p]),
    "gtn_multidot_noalloc": (_i, [_p, _i64, _i, _p, _i64, _p, _p]),
    "gtn_selftest_wait": (_i, [_p, _i64]),
    "gtn_tc_tuning": (_i, [_i, _i]),
    "gtn_tensor_create": (_i, [_p, _i, _pi64, C.POINTER(_p)]),
    "gtn_tensor_wrap": (_i, [_p, _i, _pi64, _p, C.POINTER(_p)]),
    "gtn_tensor_destroy": (_i, [_p]),
    "gtn_tensor_data": (_p, [_p]),
    "gtn_tensor_shape": (_i, [_p, _pi, _pi64]),
    "gtn_tensor_upload": (_i, [_p, _p, _i64]),
    "gtn_tensor_download": (_i, [_p, _p, _i64]),
    "gtn_site_labels": (_i, [_p, _i, _pi, _pi, _pi, _pi]),
    "gtn_map_create_kind": (_i, [_p, _p, _i, C.POINTER(_p), _i, C.POINTER(_p)]),
    "gtn_env_build": (_i, [_p, _p, _p, _p, _i, C.POINTER(_p), _p, _i]),
    "gtn_tc_tune_report": (_i, [C.c_char_p, _i64, _pi64]),
}

MAP_H1, MAP_H2, MAP_H0, MAP_ENV = 1, 2, 3, 4


class SiteDesc(C.Structure):
    """gtn_site_desc: a node's (or edge's) local structure for the kind-based calls."""
    _fields_ = [("kind", C.c_int), ("n_children", C.c_int), ("n_is_root", C.c_int), ("m_children", C.c_int),
                ("slot", C.c_int), ("m_is_root", C.c_int), ("col_major", C.c_int)]


def site_labels(desc):
    """(labels per operand, order) of a site description, from the library (no device)."""
    n = C.c_int()
    cap = 512
    ranks, labs, order = (C.c_int * 64)(), (C.c_int * cap)(), (C.c_int * 64)()
    check(lib().gtn_site_labels(C.byref(desc), cap, C.byref(n), ranks, labs, order))
    out, o = [], 0
    for i in range(n.value):
        out.append([labs[o + j] for j in range(ranks[i])])
        o += ranks[i]
    return out, [order[i] for i in range(n.value)]


TC_VARIANTS = {"ps32": 0, "ps64": 1, "ps128": 2, "ps128x2": 3, "ps256": 4, "pair256": 5, "persist128": 6,
               "persist256": 7}


class GraftError(RuntimeError):
    """Base class of library errors."""


class SpaceMismatch(ValueError):
    """Leg dimensions do not match (the reference's TensorKit.SpaceMismatch)."""


class MemoryAdmissionError(MemoryError):
    """The library refused an allocation before launching anything."""


class DeviceTimeoutError(GraftError):
    """A bounded device-side wait gave up."""


class NotConvergedError(GraftError):
    pass


def _load():
    if not os.path.exists(LIB_PATH):
        raise ImportError(f"libgrafttn.so not built at {LIB_PATH}: run __graft_entry__.build()")
    lib = C.CDLL(LIB_PATH)
    for name, (res, args) in SIGNATURES.items():
        f = getattr(lib, name)
        f.restype = res
        f.argtypes = args
    return lib


_LIB = None


def lib():
    global _LIB
    if _LIB is None:
        _LIB = _load()
    return _LIB


def check(status, ctx=None, what=""):
    if status == GTN_OK:
        return
    msg = ""
    if ctx is not None:
        raw = lib().gtn_last_error(ctx)
        msg = raw.decode() if raw else ""
    text = f"{what}: {msg}" if what else msg
    if status == GTN_ERR_INVALID:
        raise ValueError(text)
    if status == GTN_ERR_SHAPE:
        raise SpaceMismatch(text)
    if status == GTN_ERR_MEMORY:
        raise MemoryAdmissionError(text)
    if status == GTN_ERR_TIMEOUT:
        raise DeviceTimeoutError(text)
    if status == GTN_ERR_UNSUPPORTED:
        raise NotImplementedError(text)
    if status == GTN_ERR_NOT_CONVERGED:
        raise NotConvergedError(text)
    raise GraftError(f"status {status}: {text}")


def int_array(vals):
    vals = list(vals)
    return (C.c_int * max(len(vals), 1))(*vals)


def i64_array(vals):
    vals = list(vals)
    return (C.c_int64 * max(len(vals), 1))(*vals)


def ptr_array(vals):
    vals = list(vals)
    return (C.c_void_p * max(len(vals), 1))(*[C.c_void_p(v) if v else None for v in vals])


class BlockGather(C.Structure):
    _fields_ = [("src_buf", C.c_int32), ("dst_index", C.c_int32), ("ng_m", C.c_int32), ("ng_k", C.c_int32),
                ("src_off", C.c_int64), ("row_off", C.c_int64), ("col_off", C.c_int64),
                ("M", C.c_int64), ("K", C.c_int64), ("Kw", C.c_int64), ("ld", C.c_int64),
                ("m_dim", C.c_int64 * 8), ("m_str", C.c_int64 * 8), ("k_dim", C.c_int64 * 8),
                ("k_str", C.c_int64 * 8)]


class BlockGemm(C.Structure):
    _fields_ = [("b_index", C.c_int32), ("c_buf", C.c_int32), ("c_off", C.c_int64), ("M", C.c_int64),
                ("N", C.c_int64), ("K", C.c_int64)]


def tc_tuning(mode=-1, clear=False):
    """Tile-shape selection of the tensor-core steps: 'ladder' (fixed rule), 'measured'
    (default: the first launch of each problem class times every candidate and caches the
    fastest) or a variant name of TC_VARIANTS to force it; None keeps the mode.  clear
    forgets the cached choices.  Returns the previous mode as an int."""
    if mode is None or mode == -1:
        code = -1
    elif mode == "ladder":
        code = 0
    elif mode == "measured":
        code = 1
    elif isinstance(mode, str):
        code = 2 + TC_VARIANTS[mode]
    else:
        code = int(mode)
    old = lib().gtn_tc_tuning(code, 1 if clear else 0)
    if old < 0:
        raise ValueError(f"tc_tuning: bad mode {mode!r}")
    return old


def tc_tune_report():
    """The cached tile-shape choices, one text line per problem class."""
    need = C.c_int64()
    lib().gtn_tc_tune_report(None, 0, C.byref(need))
    buf = C.create_string_buffer(int(need.value) + 64)
    check(lib().gtn_tc_tune_report(buf, len(buf), C.byref(need)))
    return [l for l in buf.value.decode().split("\n") if l]
