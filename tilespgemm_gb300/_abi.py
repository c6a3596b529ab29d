"""ctypes declarations of the C ABI in include/tilespgemm.h.

The library is the in-tree ``tilespgemm_gb300/_lib/libtilespgemm.so``; loading
fails loudly when it has not been built (there is no CPU fallback).
"""
from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

LIB_PATH = Path(__file__).resolve().parent / "_lib" / "libtilespgemm.so"

# tsg_status
OK = 0
ERR_INVALID_ARG = 1
ERR_CUDA = 2
ERR_OOM = 3
ERR_INT32_OVERFLOW = 4
ERR_BAD_MTX = 5
ERR_DEVICE_TIMEOUT = 6
ERR_SHAPE = 7
ERR_BAD_INPUT = 8
ERR_NOT_SUPPORTED = 9
ERR_BUDGET = 10

# largest row count of tsg_tiles_to_csr_noalloc
NOALLOC_MAX_ROWS = 1 << 20

STATUS_NAMES = {
    0: "TSG_OK", 1: "TSG_ERR_INVALID_ARG", 2: "TSG_ERR_CUDA", 3: "TSG_ERR_OOM",
    4: "TSG_ERR_INT32_OVERFLOW", 5: "TSG_ERR_BAD_MTX", 6: "TSG_ERR_DEVICE_TIMEOUT",
    7: "TSG_ERR_SHAPE", 8: "TSG_ERR_BAD_INPUT", 9: "TSG_ERR_NOT_SUPPORTED", 10: "TSG_ERR_BUDGET",
}

# tsg_op
OP_AB, OP_AA, OP_AAT = 0, 1, 2
# tsg_mem
MEM_HOST, MEM_DEVICE = 0, 1


class tsg_csr(C.Structure):
    _fields_ = [
        ("m", C.c_int32), ("n", C.c_int32), ("nnz", C.c_int64),
        ("rowptr_bits", C.c_int32), ("where", C.c_int32),
        ("row_ptr", C.c_void_p), ("col", C.c_void_p), ("val", C.c_void_p),
        ("owner", C.c_void_p),
    ]


class tsg_opts(C.Structure):
    _fields_ = [
        ("validate", C.c_int32), ("phase_times", C.c_int32), ("out_rowptr_bits", C.c_int32),
        ("dense_tile_min", C.c_int32), ("smem_acc_max", C.c_int32), ("threads_numeric", C.c_int32),
        ("row_acc_max", C.c_int32), ("numeric_walk", C.c_int32),
        ("rows_global", C.c_int32), ("row_warps", C.c_int32), ("count_products", C.c_int32),
        ("small_path", C.c_int32),
    ]


class tsg_stats(C.Structure):
    _fields_ = [
        ("nnz_a", C.c_int64), ("nnz_b", C.c_int64), ("nnz_c", C.c_int64), ("nnz_cub", C.c_int64),
        ("tiles_a", C.c_int64), ("tiles_b", C.c_int64), ("tiles_c", C.c_int64),
        ("ms_total", C.c_double), ("ms_convert", C.c_double), ("ms_step1", C.c_double),
        ("ms_step2", C.c_double), ("ms_step3", C.c_double), ("ms_h2d", C.c_double), ("ms_d2h", C.c_double),
        ("n_syncs", C.c_int32), ("bins", C.c_int32 * 4), ("small_path", C.c_int32),
    ]

    def as_dict(self) -> dict:
        d = {f: getattr(self, f) for f, _ in self._fields_ if f != "bins"}
        d["bins"] = list(self.bins)
        return d


class tsg_tiles(C.Structure):
    _fields_ = [
        ("m", C.c_int32), ("n", C.c_int32), ("blkm", C.c_int32), ("blkn", C.c_int32),
        ("numblk", C.c_int64), ("nnz", C.c_int64),
        ("blkrowptr", C.c_void_p), ("blkcolidx", C.c_void_p), ("nnzb", C.c_void_p),
        ("ptr", C.c_void_p), ("col", C.c_void_p), ("val", C.c_void_p), ("mask", C.c_void_p),
        ("owner", C.c_void_p),
    ]


class tsg_server_opts(C.Structure):
    _fields_ = [("device", C.c_int32), ("workers", C.c_int32), ("max_batch", C.c_int32),
                ("budget_bytes", C.c_int64), ("plan_cache_bytes", C.c_int64)]


class tsg_server_result(C.Structure):
    _fields_ = [("latency_ms", C.c_double), ("queue_ms", C.c_double), ("run_ms", C.c_double),
                ("numeric_only", C.c_int32), ("batched_with", C.c_int32), ("worker", C.c_int32)]

    def as_dict(self) -> dict:
        return {f: getattr(self, f) for f, _ in self._fields_}


# name -> (restype, argtypes); the list every consumer of the ABI checks against
SIGNATURES = {
    "tsg_opts_default": (None, [C.POINTER(tsg_opts)]),
    "tsg_create": (C.c_int, [C.POINTER(C.c_void_p), C.c_int, C.POINTER(tsg_opts)]),
    "tsg_destroy": (C.c_int, [C.c_void_p]),
    "tsg_last_error": (C.c_char_p, []),
    "tsg_version": (C.c_char_p, []),
    "tsg_launch_count": (C.c_int64, []),
    "tsg_pinned_cache_cap": (C.c_int64, []),
    "tsg_get_stream": (C.c_void_p, [C.c_void_p]),
    "tsg_stream_wait": (C.c_int, [C.c_void_p, C.c_void_p]),
    "tsg_measure_fp64_peak": (C.c_int, [C.c_void_p, C.POINTER(C.c_double)]),
    "tsg_load_mtx": (C.c_int, [C.c_char_p, C.POINTER(tsg_csr), C.POINTER(C.c_int32)]),
    "tsg_load_mtx_device": (C.c_int, [C.c_void_p, C.c_char_p, C.POINTER(tsg_csr), C.POINTER(C.c_int32)]),
    "tsg_csr_free": (C.c_int, [C.c_void_p, C.POINTER(tsg_csr)]),
    "tsg_write_mtx": (C.c_int, [C.c_char_p, C.POINTER(tsg_csr), C.c_int32]),
    "tsg_spgemm": (C.c_int, [C.c_void_p, C.c_int, C.POINTER(tsg_csr), C.POINTER(tsg_csr),
                             C.POINTER(tsg_csr), C.POINTER(tsg_stats)]),
    "tsg_spgemm_batched": (C.c_int, [C.c_void_p, C.c_int, C.c_int32, C.POINTER(tsg_csr), C.POINTER(tsg_csr),
                                     C.POINTER(tsg_csr), C.POINTER(tsg_stats)]),
    "tsg_plan_create": (C.c_int, [C.c_void_p, C.c_int, C.POINTER(tsg_csr), C.POINTER(tsg_csr),
                                  C.POINTER(C.c_void_p), C.POINTER(tsg_stats)]),
    "tsg_plan_execute": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int32,
                                   C.POINTER(tsg_csr), C.POINTER(tsg_stats)]),
    "tsg_plan_nnz": (C.c_int64, [C.c_void_p]),
    "tsg_plan_device_bytes": (C.c_int64, [C.c_void_p]),
    "tsg_plan_destroy": (C.c_int, [C.c_void_p, C.c_void_p]),
    "tsg_plan_create_batched": (C.c_int, [C.c_void_p, C.c_int, C.c_int32, C.POINTER(tsg_csr), C.POINTER(tsg_csr),
                                          C.POINTER(C.c_void_p), C.POINTER(tsg_stats)]),
    "tsg_plan_count": (C.c_int32, [C.c_void_p]),
    "tsg_plan_value_offsets": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p]),
    "tsg_plan_set_values": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int32]),
    "tsg_plan_replay": (C.c_int, [C.c_void_p, C.c_void_p]),
    "tsg_plan_result": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int32, C.POINTER(tsg_csr)]),
    "tsg_plan_tune": (C.c_int, [C.c_void_p, C.c_void_p, C.POINTER(C.c_double)]),
    "tsg_server_opts_default": (None, [C.POINTER(tsg_server_opts)]),
    "tsg_server_create": (C.c_int, [C.POINTER(tsg_server_opts), C.POINTER(C.c_void_p)]),
    "tsg_server_submit": (C.c_int, [C.c_void_p, C.c_int, C.POINTER(tsg_csr), C.POINTER(tsg_csr), C.c_uint64,
                                    C.POINTER(C.c_int64)]),
    "tsg_server_wait": (C.c_int, [C.c_void_p, C.c_int64, C.POINTER(tsg_csr), C.POINTER(tsg_server_result)]),
    "tsg_server_wait_any": (C.c_int, [C.c_void_p, C.POINTER(C.c_int64), C.POINTER(tsg_csr),
                                      C.POINTER(tsg_server_result)]),
    "tsg_server_destroy": (C.c_int, [C.c_void_p]),
    "tsg_csr_to_tiles": (C.c_int, [C.c_void_p, C.POINTER(tsg_csr), C.POINTER(tsg_tiles)]),
    "tsg_spgemm_tiles": (C.c_int, [C.c_void_p, C.c_int, C.POINTER(tsg_csr), C.POINTER(tsg_csr),
                                   C.POINTER(tsg_tiles), C.POINTER(tsg_stats)]),
    "tsg_tiles_to_csr": (C.c_int, [C.c_void_p, C.POINTER(tsg_tiles), C.POINTER(tsg_csr)]),
    "tsg_tiles_free": (C.c_int, [C.c_void_p, C.POINTER(tsg_tiles)]),
    "tsg_tiles_spmv": (C.c_int, [C.c_void_p, C.POINTER(tsg_tiles), C.c_void_p, C.c_void_p]),
    "tsg_tiles_to_csr_noalloc": (C.c_int, [C.c_void_p, C.POINTER(tsg_tiles), C.c_void_p, C.c_void_p, C.c_void_p]),
    "tsg_tiles_download": (C.c_int, [C.c_void_p, C.POINTER(tsg_tiles), C.c_void_p, C.c_void_p, C.c_void_p,
                                     C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
    "tsg_csr_download": (C.c_int, [C.c_void_p, C.POINTER(tsg_csr), C.c_void_p, C.c_void_p, C.c_void_p]),
    "tsg_plan_settings": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
    "tsg_inject_alloc_failure": (C.c_int, [C.c_int32, C.c_int64]),
    "tsg_alloc_failure_pending": (C.c_int64, [C.c_int32]),
    "tsg_check_bounded_wait": (C.c_int, [C.c_void_p, C.c_int64, C.c_int32]),
    "tsg_csr_to_device": (C.c_int, [C.c_void_p, C.POINTER(tsg_csr), C.POINTER(tsg_csr)]),
    "tsg_csr_download_rows": (C.c_int, [C.c_void_p, C.POINTER(tsg_csr), C.c_int32, C.c_int32, C.c_void_p,
                                        C.c_void_p, C.c_void_p]),
}

_lib = None


class TSGError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(f"{STATUS_NAMES.get(status, status)}: {msg}")
        self.status = status


def lib() -> C.CDLL:
    """Load libtilespgemm.so (RTLD_GLOBAL not needed; the CUDA runtime is static)."""
    global _lib
    if _lib is None:
        path = Path(os.environ.get("TSG_LIB", LIB_PATH))
        if not path.exists():
            raise RuntimeError(
                f"{path} is missing: build it with `python -c 'import __graft_entry__ as g; g.build()'` "
                "(nvcc, sm_103a). There is no CPU fallback.")
        handle = C.CDLL(str(path))
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(handle, name)
            fn.restype = res
            fn.argtypes = args
        _lib = handle
    return _lib


def check(status: int) -> None:
    if status != OK:
        msg = lib().tsg_last_error().decode(errors="replace")
        raise TSGError(status, msg)
