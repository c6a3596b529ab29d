"""tilespgemm_gb300 -- GB300-native (sm_103a) tiled FP64 SpGEMM.

A drop-in for the SpGEMM call of YuyaoNiu/TileSpGEMM: CSR in, CSR out, FP64
values, 32-bit column indices, the reference's Matrix Market load path.  The
compute path is hand-written CUDA in libtilespgemm.so behind the C ABI of
include/tilespgemm.h; this package is the Python host-side mirror of it.
"""
from .api import (CSR, Context, OwnedCSR, Plan, Tiles, TSGError, load_mtx, pinned_cache_cap,  # noqa: F401
                  version, write_mtx)

__all__ = ["CSR", "Context", "OwnedCSR", "Plan", "Tiles", "TSGError", "load_mtx", "write_mtx", "version",
           "pinned_cache_cap"]
