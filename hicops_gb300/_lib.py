"""ctypes binding of libhicops_gb300.so (include/hicops_gb300.h).

The library is the only compute path: if it is missing, or no sm_103 device
is present, every call raises — there is no CPU fallback.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libhicops_gb300.so")

HC_HIST_BINS = 1002
HC_QALEN = 100
HC_MAX_MODS = 15

STATUS = {0: "success", -3001: "invalid memory", -3002: "invalid parameter", -3003: "invalid index",
          -3004: "invalid size", -3007: "allocation failed", -3008: "invalid pointer",
          -3010: "invalid modification", -3012: "not enough data", -3006: "file not found",
          -3013: "file error", -3020: "CUDA error",
          -3021: "work still running at the deadline", -3022: "no usable CUDA device"}

ENTRY_DTYPE = np.dtype([("mass", "<f4"), ("seqid", "<u4"), ("sites", "<u8"),
                        ("modnum", "<u4"), ("pad", "<u4")])
RESULT_DTYPE = np.dtype([
    ("cpsms", "<u4"), ("idxoffset", "<i4"), ("psid", "<i4"), ("sharedions", "<u2"),
    ("totalions", "<u2"), ("hyperscore", "<f4"), ("mu", "<i4"), ("beta", "<i4"),
    ("minhyp", "<i4"), ("nexthyp", "<i4"), ("maxhyp", "<i4"), ("flags", "<u4"),
    ("reported", "<u4"), ("evalue", "<f8"), ("post_bytes", "<u8")])
assert ENTRY_DTYPE.itemsize == 24 and RESULT_DTYPE.itemsize == 64

FLAG_LGFACT_OOB, FLAG_HIST_OOB, FLAG_TAILFIT_OOB, FLAG_TAILFIT_EMPTY, FLAG_WIDE = 1, 2, 4, 8, 0x100
FLAG_LEARNED = 0x200


class HcParams(C.Structure):
    _fields_ = [("min_len", C.c_uint32), ("max_len", C.c_uint32), ("maxz", C.c_uint32),
                ("topmatches", C.c_uint32), ("scale", C.c_uint32), ("min_shp", C.c_uint32),
                ("min_cpsm", C.c_uint32), ("min_mass", C.c_uint32), ("max_mass", C.c_uint32),
                ("dF", C.c_uint32), ("base_int", C.c_int32), ("min_int", C.c_int32),
                ("dM", C.c_double), ("expect_max", C.c_double), ("nmods", C.c_uint32),
                ("vmods_per_pep", C.c_uint32), ("mod_mass", C.c_uint32 * HC_MAX_MODS),
                ("mod_res", (C.c_char * 4) * HC_MAX_MODS), ("mod_per_pep", C.c_uint32 * HC_MAX_MODS),
                ("threads", C.c_uint32)]


class HcTuning(C.Structure):
    _fields_ = [("threads", C.c_uint32), ("tile", C.c_uint32), ("ctas_per_sm", C.c_uint32),
                ("pairs_per_warp", C.c_uint32), ("schedule", C.c_uint32), ("defer_cap", C.c_uint32),
                ("small_log2", C.c_uint32)]


def to_hc_params(p) -> HcParams:
    c = HcParams()
    for k in ("min_len", "max_len", "maxz", "topmatches", "scale", "min_shp", "min_cpsm",
              "min_mass", "max_mass", "dF", "base_int", "min_int", "vmods_per_pep", "threads"):
        setattr(c, k, int(getattr(p, k)))
    c.dM = float(p.dM)
    c.expect_max = float(p.expect_max)
    c.nmods = len(p.mods)
    for i, (res, _mass, per) in enumerate(p.mods):
        c.mod_mass[i] = p.mod_mass_scaled(i)
        c.mod_res[i].value = res.encode()[:4]
        c.mod_per_pep[i] = int(per)
    return c


_lib = None

# (name, restype, argtypes)
_SIGS = [
    ("hc_version", C.c_int, []),
    ("hc_status_string", C.c_char_p, [C.c_int]),
    ("hc_ctx_create", C.c_int, [C.c_int, C.POINTER(HcParams), C.POINTER(C.c_void_p)]),
    ("hc_ctx_destroy", C.c_int, [C.c_void_p]),
    ("hc_last_error", C.c_char_p, [C.c_void_p]),
    ("hc_ctx_set_tuning", C.c_int, [C.c_void_p, C.POINTER(HcTuning)]),
    ("hc_ctx_get_tuning", C.c_int, [C.c_void_p, C.POINTER(HcTuning)]),
    ("hc_ctx_wait", C.c_int, [C.c_void_p, C.c_void_p, C.c_double]),
    ("hc_dslim_construct", C.c_int, [C.c_void_p, C.c_uint32, C.c_void_p, C.c_uint32, C.c_void_p, C.c_uint32]),
    ("hc_dslim_load", C.c_int, [C.c_void_p, C.c_uint32, C.c_void_p, C.c_uint32, C.c_void_p, C.c_uint32,
                                C.c_void_p, C.c_void_p]),
    ("hc_dslim_info", C.c_int, [C.c_void_p, C.c_uint32, C.POINTER(C.c_uint32), C.POINTER(C.c_uint64)]),
    ("hc_dslim_export", C.c_int, [C.c_void_p, C.c_uint32, C.c_void_p, C.c_void_p, C.c_void_p]),
    ("hc_make_entries", C.c_int64, [C.POINTER(HcParams), C.c_uint32, C.c_void_p, C.c_uint32, C.c_void_p,
                                    C.c_int64]),
    ("hc_dslim_query", C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                 C.c_uint32, C.c_void_p, C.c_void_p]),
    ("hc_dslim_save", C.c_int, [C.c_void_p, C.c_char_p]),
    ("hc_dslim_restore", C.c_int, [C.c_void_p, C.c_char_p]),
    ("hc_write_psms", C.c_int, [C.c_void_p, C.c_char_p, C.c_char_p, C.c_uint32, C.c_void_p, C.c_uint32,
                                C.c_void_p, C.c_void_p, C.c_void_p, C.c_int]),
    ("hc_ms2_open", C.c_int, [C.c_void_p, C.c_char_p, C.POINTER(C.c_void_p), C.POINTER(C.c_uint32),
                              C.POINTER(C.c_uint32)]),
    ("hc_ms2_extract", C.c_int, [C.c_void_p, C.c_void_p, C.c_uint32, C.c_uint32, C.c_void_p, C.c_void_p,
                                 C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.POINTER(C.c_uint32),
                                 C.POINTER(C.c_uint64)]),
    ("hc_ms2_close", C.c_int, [C.c_void_p]),
    ("hc_ms2_read", C.c_int, [C.c_char_p, C.c_uint32, C.POINTER(C.c_void_p), C.POINTER(C.c_uint32),
                              C.POINTER(C.c_uint32)]),
    ("hc_ms2_raw", C.c_int, [C.c_void_p, C.c_uint32, C.c_uint32, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                             C.c_void_p, C.c_void_p]),
    ("hc_dslim_query_stream", C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                        C.c_uint32, C.c_uint32, C.c_void_p, C.c_void_p, C.c_void_p,
                                        C.c_void_p]),
    ("hc_dslim_query_device", C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                        C.c_void_p, C.c_uint32, C.c_uint32, C.c_void_p, C.c_void_p,
                                        C.c_void_p]),
    ("hc_last_launch_count", C.c_int, [C.c_void_p]),
    ("hc_check_division", C.c_uint64, [C.c_uint32, C.c_uint32]),
    ("hc_ctx_set_phase_timing", C.c_int, [C.c_void_p, C.c_int]),
    ("hc_mlp_create", C.c_int, [C.c_void_p, C.c_uint64, C.POINTER(C.c_void_p)]),
    ("hc_mlp_destroy", C.c_int, [C.c_void_p]),
    ("hc_mlp_num_params", C.c_int, []),
    ("hc_mlp_get_params", C.c_int, [C.c_void_p, C.c_void_p]),
    ("hc_mlp_set_params", C.c_int, [C.c_void_p, C.c_void_p]),
    ("hc_mlp_features", C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_uint32, C.c_void_p, C.c_void_p]),
    ("hc_mlp_targets", C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_uint32, C.c_void_p, C.c_void_p]),
    ("hc_mlp_forward", C.c_int, [C.c_void_p, C.c_void_p, C.c_uint32, C.c_void_p, C.c_void_p]),
    ("hc_mlp_gradients", C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_uint32, C.c_void_p,
                                   C.POINTER(C.c_float)]),
    ("hc_mlp_train", C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_uint32, C.c_uint32, C.c_uint32, C.c_float,
                               C.POINTER(C.c_float)]),
    ("hc_mlp_set_gate", C.c_int, [C.c_void_p, C.c_float, C.c_uint32]),
    ("hc_mlp_get_gate", C.c_int, [C.c_void_p, C.POINTER(C.c_float), C.POINTER(C.c_uint32)]),
    ("hc_mlp_tail_probe", C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_uint32, C.c_int,
                                    C.c_void_p, C.c_void_p, C.c_void_p]),
    ("hc_dslim_query_learned", C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                         C.c_void_p, C.c_uint32, C.c_uint32, C.c_void_p, C.c_void_p, C.c_void_p,
                                         C.c_void_p]),
    ("hc_phase_cycles", C.c_int, [C.c_void_p, C.POINTER(C.c_uint64)]),
    ("hc_dslim_query_graph", C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                       C.c_void_p, C.c_uint32, C.c_uint32, C.c_void_p, C.c_void_p,
                                       C.c_void_p]),
    ("hc_dslim_query_noalloc", C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                         C.c_void_p, C.c_uint32, C.c_uint32, C.c_void_p, C.c_void_p,
                                         C.c_void_p]),
    ("hc_tune", C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_uint32,
                          C.c_uint32, C.c_void_p, C.c_void_p, C.c_void_p, C.POINTER(C.c_float)]),
    ("hc_ctx_set_profiling", C.c_int, [C.c_void_p, C.c_int]),
    ("hc_last_stage_times", C.c_int, [C.c_void_p, C.POINTER(C.c_float), C.POINTER(C.c_int)]),
    ("hc_last_kernel_times", C.c_int, [C.c_void_p, C.POINTER(C.c_float), C.POINTER(C.c_float),
                                       C.POINTER(C.c_float), C.POINTER(C.c_float)]),
]

EXPORTED = [s[0] for s in _SIGS]


def load(path: str | None = None):
    """Load the library (raises when it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    path = path or LIB_PATH
    if not os.path.exists(path):
        raise RuntimeError(f"{path} is missing: build it with `python -m hicops_gb300.build` "
                           "(there is no CPU fallback)")
    lib = C.CDLL(path)
    for name, res, args in _SIGS:
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


class HcError(RuntimeError):
    def __init__(self, status: int, what: str, detail: str = ""):
        super().__init__(f"{what}: {STATUS.get(status, status)} ({status}) {detail}".strip())
        self.status = status


def ptr(a) -> C.c_void_p | None:
    if a is None:
        return None
    if isinstance(a, int):
        return C.c_void_p(a)
    return C.c_void_p(a.ctypes.data)
