"""ctypes bindings of the C ABI declared in include/cosma_gb300.h.

The shared library is built in-tree (cosma_gb300/_lib/libcosma_gb300.so).
There is no fallback: if the library is missing or fails to load, every
entry point raises.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

LIB_PATH = Path(__file__).resolve().parent / "_lib" / "libcosma_gb300.so"

SUCCESS = 0
METHOD_AUTO, METHOD_NATIVE, METHOD_OZAKI, METHOD_BF16X3, METHOD_OZAKI2 = 0, 1, 2, 3, 4
METHODS = {"auto": METHOD_AUTO, "native": METHOD_NATIVE, "ozaki": METHOD_OZAKI, "bf16x3": METHOD_BF16X3,
           "ozaki2": METHOD_OZAKI2}


class CosmaGpuError(RuntimeError):
    def __init__(self, code: int, message: str):
        super().__init__(f"cosma_gb300 error {code}: {message}")
        self.code = code


class OzakiInfo(C.Structure):
    _fields_ = [("slices", C.c_int), ("products", C.c_int), ("groups", C.c_int), ("fallback_native", C.c_int),
                ("spread_bits", C.c_double), ("prep_ms", C.c_double), ("gemm_ms", C.c_double),
                ("fraction_bits", C.c_int), ("exact_product", C.c_int)]

    def as_dict(self):
        return {f: getattr(self, f) for f, _ in self._fields_}


class GemmProblem(C.Structure):
    _fields_ = [("transa", C.c_char), ("transb", C.c_char), ("m", C.c_int32), ("n", C.c_int32), ("k", C.c_int32),
                ("alpha", C.c_double), ("beta", C.c_double), ("A", C.c_void_p), ("lda", C.c_int64),
                ("B", C.c_void_p), ("ldb", C.c_int64), ("C", C.c_void_p), ("ldc", C.c_int64)]


class GroupedInfo(C.Structure):
    _fields_ = [("tiles", C.c_int), ("tile_policy", C.c_int), ("dynamic_schedule", C.c_int),
                ("warps_per_cta", C.c_int), ("useful_flops", C.c_double), ("padded_flops", C.c_double),
                ("tuned_ms", C.c_double)]

    def as_dict(self):
        return {f: getattr(self, f) for f, _ in self._fields_}


class Block(C.Structure):  # cosma_gpu_block (the reference's `block`)
    _fields_ = [("data", C.c_void_p), ("ld", C.c_int), ("row", C.c_int), ("col", C.c_int)]


class Layout(C.Structure):  # cosma_gpu_layout (the reference's `layout`)
    _fields_ = [("rowblocks", C.c_int), ("colblocks", C.c_int), ("rowsplit", C.POINTER(C.c_int)),
                ("colsplit", C.POINTER(C.c_int)), ("owners", C.POINTER(C.c_int)), ("nlocalblocks", C.c_int),
                ("localblocks", C.POINTER(Block))]


i32, i64, dbl, flt, vp, ch = C.c_int, C.c_int64, C.c_double, C.c_float, C.c_void_p, C.c_char
_PX = [vp] * 19

SIGNATURES = {
    "cosma_gpu_last_error": (i32, []),
    "cosma_gpu_last_error_string": (C.c_char_p, []),
    "cosma_gpu_version": (C.c_char_p, []),
    "cosma_gpu_tmm_make_context": (vp, [ch, i32, i32, i32, i32]),
    "cosma_gpu_tmm_destroy_context": (None, [vp]),
    "cosma_gpu_tmm_set_method": (i32, [vp, i32, i32]),
    "cosma_gpu_tmm_device_buffer_c": (vp, [vp]),
    "cosma_gpu_tmm_last_ozaki_info": (i32, [vp, C.POINTER(OzakiInfo)]),
    "cosma_gpu_tmm_last_transfer_bytes": (i32, [vp, C.POINTER(C.c_int64), C.POINTER(C.c_int64)]),
    "cosma_gpu_tmm_last_overlapped": (i32, [vp]),
    "cosma_gpu_tmm_tiles_for_memory": (i32, [ch, i32, i64, C.POINTER(C.c_int), C.POINTER(C.c_int),
                                             C.POINTER(C.c_int)]),
    "cosma_gpu_tmm_set_memory_limit": (i32, [vp, i64]),
    "cosma_gpu_tmm_tiles": (i32, [vp, C.POINTER(C.c_int), C.POINTER(C.c_int), C.POINTER(C.c_int)]),
    "cosma_gpu_tmm_gemm_s": (i32, [vp, ch, ch, i32, i32, i32, flt, vp, i32, vp, i32, flt, vp, i32, i32, i32]),
    "cosma_gpu_tmm_gemm_d": (i32, [vp, ch, ch, i32, i32, i32, dbl, vp, i32, vp, i32, dbl, vp, i32, i32, i32]),
    "cosma_gpu_tmm_gemm_c": (i32, [vp, ch, ch, i32, i32, i32, vp, vp, i32, vp, i32, vp, vp, i32, i32, i32]),
    "cosma_gpu_tmm_gemm_z": (i32, [vp, ch, ch, i32, i32, i32, vp, vp, i32, vp, i32, vp, vp, i32, i32, i32]),
    "cosma_gpu_local_multiply_s": (i32, [vp, vp, vp, vp, i32, i32, i32, flt, flt, i32]),
    "cosma_gpu_local_multiply_d": (i32, [vp, vp, vp, vp, i32, i32, i32, dbl, dbl, i32]),
    "cosma_gpu_local_multiply_c": (i32, [vp, vp, vp, vp, i32, i32, i32, vp, vp, i32]),
    "cosma_gpu_local_multiply_z": (i32, [vp, vp, vp, vp, i32, i32, i32, vp, vp, i32]),
    "cosma_gpu_context_instance": (vp, [ch]),
    "cosma_gpu_selftest_wait_timeout": (i32, [C.c_ulonglong, vp]),
    "cosma_gpu_smultiply_using_layout": (i32, [C.c_char_p, C.c_char_p, vp, C.POINTER(Layout), C.POINTER(Layout), vp,
                                               C.POINTER(Layout)]),
    "cosma_gpu_dmultiply_using_layout": (i32, [C.c_char_p, C.c_char_p, vp, C.POINTER(Layout), C.POINTER(Layout), vp,
                                               C.POINTER(Layout)]),
    "cosma_gpu_cmultiply_using_layout": (i32, [C.c_char_p, C.c_char_p, vp, C.POINTER(Layout), C.POINTER(Layout), vp,
                                               C.POINTER(Layout)]),
    "cosma_gpu_zmultiply_using_layout": (i32, [C.c_char_p, C.c_char_p, vp, C.POINTER(Layout), C.POINTER(Layout), vp,
                                               C.POINTER(Layout)]),
    "cosma_gpu_dgemm_device": (i32, [i32, ch, ch, i64, i64, i64, dbl, vp, i64, vp, i64, dbl, vp, i64, vp]),
    "cosma_gpu_zgemm_device": (i32, [i32, ch, ch, i64, i64, i64, vp, vp, i64, vp, i64, vp, vp, i64, vp]),
    "cosma_gpu_sgemm_device": (i32, [i32, ch, ch, i64, i64, i64, flt, vp, i64, vp, i64, flt, vp, i64, vp]),
    "cosma_gpu_cgemm_device": (i32, [i32, ch, ch, i64, i64, i64, vp, vp, i64, vp, i64, vp, vp, i64, vp]),
    "cosma_gpu_dgemm_ozaki_device": (i32, [ch, ch, i64, i64, i64, dbl, vp, i64, vp, i64, dbl, vp, i64, i32, vp,
                                           C.POINTER(OzakiInfo)]),
    "cosma_gpu_zgemm_ozaki_device": (i32, [ch, ch, i64, i64, i64, vp, vp, i64, vp, i64, vp, vp, i64, i32, vp,
                                           C.POINTER(OzakiInfo)]),
    "cosma_gpu_dgemm_ozaki2_device": (i32, [ch, ch, i64, i64, i64, dbl, vp, i64, vp, i64, dbl, vp, i64, i32, vp,
                                            C.POINTER(OzakiInfo)]),
    "cosma_gpu_zgemm_ozaki2_device": (i32, [ch, ch, i64, i64, i64, vp, vp, i64, vp, i64, vp, vp, i64, i32, vp,
                                            C.POINTER(OzakiInfo)]),
    "cosma_gpu_dgemm_ozaki2_residual": (i32, [ch, ch, i64, i64, i64, vp, i64, vp, i64, vp, i64, i32, vp, vp, i64, vp,
                                              C.POINTER(OzakiInfo)]),
    "cosma_gpu_ozaki2_choose": (i32, [i64, dbl, i32, i32, C.POINTER(C.c_int), C.POINTER(C.c_int)]),
    "cosma_gpu_release_workspaces": (i32, [vp]),
    "cosma_gpu_dgemm_ozaki_noalloc": (i32, [ch, ch, i64, i64, i64, dbl, vp, i64, vp, i64, dbl, vp, i64, i32, vp,
                                            C.POINTER(OzakiInfo)]),
    "cosma_gpu_grouped_plan_create": (vp, [i32, i32, C.POINTER(GemmProblem), i32, vp]),
    "cosma_gpu_grouped_plan_run": (i32, [vp, vp]),
    "cosma_gpu_grouped_plan_info": (i32, [vp, C.POINTER(GroupedInfo)]),
    "cosma_gpu_grouped_plan_slices": (i32, [vp, C.POINTER(C.c_int)]),
    "cosma_gpu_grouped_plan_destroy": (None, [vp]),
    "cosma_gpu_dgemm_grouped_device": (i32, [i32, i32, C.POINTER(GemmProblem), vp]),
    "costa_gpu_pack": (i32, [ch, i32, i32, i64, i64, vp, i64, vp, i64, vp]),
    "costa_gpu_unpack_d": (i32, [i64, i64, dbl, vp, i64, dbl, vp, i64, vp]),
    "costa_gpu_unpack_s": (i32, [i64, i64, flt, vp, i64, flt, vp, i64, vp]),
    "costa_gpu_unpack_z": (i32, [i64, i64, vp, vp, i64, vp, vp, i64, vp]),
    "costa_gpu_unpack_c": (i32, [i64, i64, vp, vp, i64, vp, vp, i64, vp]),
    "cosma_gpu_pxgemm_set_method": (i32, [i32]),
    "cosma_gpu_pxgemm_last_transfers": (i32, [C.POINTER(i64), C.POINTER(i64), C.POINTER(C.c_int)]),
    "cosma_gpu_test_fail_next": (i32, [i32, i32]),
    "cosma_gpu_test_faults_pending": (i32, [i32]),
    "cosma_gpu_host_copy_route": (i32, [vp]),
}
for _pre in ("p", "P", "cosma_p", "COSMA_P"):
    for _t in "sdcz":
        t = _t if _pre[-1] == "p" else _t.upper()
        for _suf in ("", "_"):
            base = f"{_pre}{t}gemm" if _pre[-1] == "p" else f"{_pre}{t}GEMM"
            SIGNATURES[base + _suf] = (None, _PX)

_lib = None


def load():
    """Loads the library (building nothing); raises if it is missing."""
    global _lib
    if _lib is not None:
        return _lib
    if not LIB_PATH.exists():
        raise ImportError(f"{LIB_PATH} is missing: build it with `python -m cosma_gb300.build` "
                          "(there is no non-CUDA fallback)")
    lib = C.CDLL(str(LIB_PATH))
    for name, (res, args) in SIGNATURES.items():
        f = getattr(lib, name)
        f.restype = res
        f.argtypes = args
    _lib = lib
    return lib


def check(status: int):
    if status != SUCCESS:
        lib = load()
        raise CosmaGpuError(status, lib.cosma_gpu_last_error_string().decode(errors="replace"))
    return status
