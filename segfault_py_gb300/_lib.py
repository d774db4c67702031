"""ctypes binding of libsegfock.so (the C ABI of include/segfock.h).

The library is built in-tree by segfault_py_gb300/build.py.  There is no CPU
fallback: if the shared library is missing or cannot be loaded, every entry
point raises SegFockUnavailable.
"""
from __future__ import annotations

import ctypes as C
import os

LIB_PATH = os.path.join(os.path.dirname(os.path.abspath(__file__)), "csrc", "libsegfock.so")

SF_PREC_FP64 = 0
SF_PREC_FP32 = 1
SF_PREC_MIXED = 2
SF_PREC_MIXED_DF = 3
SF_PREC_DF = 4
PRECISION = {"fp64": SF_PREC_FP64, "fp32": SF_PREC_FP32, "mixed": SF_PREC_MIXED, "mixed_df": SF_PREC_MIXED_DF,
             "df": SF_PREC_DF}

EXPORTS = ["sf_version", "sf_last_error", "sf_create", "sf_build_shells", "sf_destroy", "sf_nao", "sf_npairs",
           "sf_schwarz", "sf_fock_jk", "sf_set_partition", "sf_eri_batch", "sf_one_electron", "sf_rys_roots_host", "sf_set_profiling", "sf_slice_count", "sf_get_slice_info",
           "sf_fma_peak", "sf_fock_jk_noalloc", "sf_grad_jk", "sf_grad_one_electron",
           "sf_small_solve", "sf_eri_plan_create", "sf_eri_plan_info", "sf_eri_plan_offsets", "sf_eri_plan_run",
           "sf_eri_plan_destroy", "sf_autotune", "sf_tuning_count", "sf_get_tuning", "sf_set_tuning", "sf_eri_plan_run_md",
           "sf_set_density_screening", "sf_set_launch_mode", "sf_fock_jk_graph_create", "sf_fock_graph_launch",
           "sf_fock_graph_destroy", "sf_debug_tc_wait_limit", "sf_grad_stats", "sf_graph_instantiate"]


class SegFockUnavailable(ImportError):
    pass


class SegFockError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__("segfock error %d: %s" % (code, msg))
        self.code = code


class ShellDesc(C.Structure):
    _fields_ = [("l", C.c_int32), ("nprim", C.c_int32), ("atom", C.c_int32), ("ao_offset", C.c_int32),
                ("center", C.c_double * 3), ("exps", C.POINTER(C.c_double)), ("coefs", C.POINTER(C.c_double))]


class Stats(C.Structure):
    _fields_ = [("quartets_fp64", C.c_int64), ("quartets_fp32", C.c_int64), ("quartets_total", C.c_int64),
                ("prim_quartets_fp64", C.c_int64), ("prim_quartets_fp32", C.c_int64),
                ("flop_alg_fp64", C.c_double), ("flop_alg_fp32", C.c_double),
                ("launches", C.c_int32), ("reserved", C.c_int32)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_ if k != "reserved"}


class SliceInfo(C.Structure):
    _fields_ = [("cls", C.c_int32), ("precision", C.c_int32), ("la", C.c_int32), ("lb", C.c_int32),
                ("lc", C.c_int32), ("ld", C.c_int32), ("quartets", C.c_int64), ("prim_quartets", C.c_int64),
                ("flop_alg", C.c_double), ("ms", C.c_float), ("threads_per_quartet", C.c_int32),
                ("start_ms", C.c_float), ("stream", C.c_int32)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class TuneEntry(C.Structure):
    _fields_ = [("cls", C.c_int32), ("precision", C.c_int32), ("cost", C.c_int64), ("split", C.c_int32),
                ("ms_default", C.c_float), ("ms_tuned", C.c_float)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


_lib = None


def lib():
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise SegFockUnavailable("libsegfock.so is not built (%s); run segfault_py_gb300/build.py" % LIB_PATH)
    try:
        L = C.CDLL(LIB_PATH)
    except OSError as e:
        raise SegFockUnavailable("cannot load %s: %s" % (LIB_PATH, e))
    p, i32, i64, d = C.c_void_p, C.c_int32, C.c_int64, C.c_double
    L.sf_version.restype = C.c_int
    L.sf_last_error.restype = C.c_char_p
    L.sf_create.argtypes = [p, i32, C.POINTER(p)]
    L.sf_build_shells.argtypes = [p, i32, C.POINTER(p)]
    L.sf_destroy.argtypes = [p]
    L.sf_destroy.restype = None
    L.sf_nao.argtypes = [p]
    L.sf_nao.restype = i32
    L.sf_npairs.argtypes = [p]
    L.sf_npairs.restype = i64
    L.sf_schwarz.argtypes = [p, p, p]
    L.sf_fock_jk.argtypes = [p, p, p, p, i32, d, d, p, p]
    L.sf_set_partition.argtypes = [p, i32, i32]
    L.sf_eri_batch.argtypes = [p, p, i64, i32, p, p, p]
    L.sf_one_electron.argtypes = [p, p, p, i32, p, p, p, p]
    L.sf_rys_roots_host.argtypes = [i32, d, i32, p, p]
    L.sf_set_profiling.argtypes = [p, i32]
    L.sf_slice_count.argtypes = [p]
    L.sf_slice_count.restype = i32
    L.sf_get_slice_info.argtypes = [p, i32, p]
    L.sf_fma_peak.argtypes = [i32, p, p, p]
    L.sf_fock_jk_noalloc.argtypes = [p, p, p, p, i32, d, d, p]
    L.sf_grad_jk.argtypes = [p, p, p, i32, d, d, p]
    L.sf_grad_one_electron.argtypes = [p, p, p, i32, p, p, p, p]
    L.sf_small_solve.argtypes = [i32, p, p, p, p, p]
    L.sf_eri_plan_create.argtypes = [p, p, i64, C.POINTER(p)]
    L.sf_eri_plan_info.argtypes = [p, p, p, p]
    L.sf_eri_plan_offsets.argtypes = [p, p]
    L.sf_eri_plan_run.argtypes = [p, i32, p, p]
    L.sf_eri_plan_run_md.argtypes = [p, i32, p, p]
    L.sf_eri_plan_destroy.argtypes = [p]
    L.sf_eri_plan_destroy.restype = None
    L.sf_autotune.argtypes = [p, p, i32, d, d, i32, p]
    L.sf_tuning_count.argtypes = [p]
    L.sf_tuning_count.restype = i32
    L.sf_get_tuning.argtypes = [p, i32, p]
    L.sf_set_tuning.argtypes = [p, p, i32]
    L.sf_set_density_screening.argtypes = [p, i32, d, d, d]
    L.sf_set_launch_mode.argtypes = [p, i32, i32]
    L.sf_fock_jk_graph_create.argtypes = [p, p, p, p, i32, d, d, i32, p, p]
    L.sf_fock_graph_launch.argtypes = [p, p]
    L.sf_fock_graph_destroy.argtypes = [p]
    L.sf_fock_graph_destroy.restype = None
    L.sf_debug_tc_wait_limit.argtypes = [i32]
    L.sf_grad_stats.argtypes = [p, p, p]
    L.sf_graph_instantiate.argtypes = [p, i32, p]
    _lib = L
    return L


def check(rc: int):
    if rc != 0:
        raise SegFockError(rc, lib().sf_last_error().decode())
