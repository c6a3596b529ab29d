"""Python host-side mirror of the reference's SpGEMM call, over the C ABI.

The reference (YuyaoNiu/TileSpGEMM) exposes its SpGEMM only through its CLI
driver (main_spgemm-col.cu:4821-5577): ``mmio_allinone`` loads a Matrix
Market file into CSR, ``AAT`` (a compile-time switch, :24) selects A*A or
A*A^T, and ``stepall_cuda_new`` runs the device pipeline and reports nnzC,
time and GFLOPS = 2*nnzCub/time (:4787).  This module offers the same
operations as calls:

    A = load_mtx("x.mtx")                       # mmio_allinone semantics
    with Context(device=0) as ctx:
        C = ctx.spgemm(A, op="AA")              # CSR in, CSR out (host)
        C, st = ctx.spgemm(A, op="AAT", stats=True)
        T = ctx.spgemm_tiles(A, op="AA")        # C in the reference's tile form

Every call goes through libtilespgemm.so; errors raise TSGError with the
library's status (the reference has no error reporting at all).
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass
from typing import Any

import numpy as np

from . import _abi
from ._abi import TSGError, check, lib

_OPS = {"AB": _abi.OP_AB, "AA": _abi.OP_AA, "AAT": _abi.OP_AAT}


@dataclass
class CSR:
    """A CSR matrix on the host (numpy) or the device (torch CUDA tensors)."""
    m: int
    n: int
    rowptr: Any          # int32 or int64, m+1
    col: Any             # int32, nnz
    val: Any             # float64, nnz

    @property
    def nnz(self) -> int:
        return int(self.col.shape[0])

    @property
    def on_device(self) -> bool:
        return hasattr(self.col, "is_cuda") and bool(self.col.is_cuda)

    @classmethod
    def from_scipy(cls, s) -> "CSR":
        s = s.tocsr()
        return cls(s.shape[0], s.shape[1], np.ascontiguousarray(s.indptr.astype(np.int64)),
                   np.ascontiguousarray(s.indices.astype(np.int32)),
                   np.ascontiguousarray(s.data.astype(np.float64)))

    def to_scipy(self):
        import scipy.sparse as sp
        return sp.csr_matrix((np.asarray(self.val), np.asarray(self.col), np.asarray(self.rowptr)),
                             shape=(self.m, self.n))

    def to_device(self, device: int = 0) -> "CSR":
        import torch
        dev = torch.device("cuda", device)
        return CSR(self.m, self.n, torch.as_tensor(np.asarray(self.rowptr)).to(dev),
                   torch.as_tensor(np.asarray(self.col)).to(dev), torch.as_tensor(np.asarray(self.val)).to(dev))

    def _tsg(self, ctx_handle=None) -> tuple[_abi.tsg_csr, list]:
        """tsg_csr view of this matrix plus the objects that must stay alive.
        Device tensors: the context's stream (ctx_handle) is ordered after
        torch's current stream without blocking; without a context the host
        waits for torch's stream."""
        s = _abi.tsg_csr()
        s.m, s.n = int(self.m), int(self.n)
        keep: list = []
        if self.on_device:
            import torch
            rp, col, val = self.rowptr, self.col, self.val
            if rp.dtype not in (torch.int32, torch.int64) or col.dtype != torch.int32 or val.dtype != torch.float64:
                raise TypeError("device CSR needs int32/int64 row pointers, int32 columns, float64 values")
            rp, col, val = rp.contiguous(), col.contiguous(), val.contiguous()
            keep += [rp, col, val]
            s.rowptr_bits = 64 if rp.dtype == torch.int64 else 32
            s.where = _abi.MEM_DEVICE
            s.row_ptr, s.col, s.val = rp.data_ptr(), col.data_ptr(), val.data_ptr()
            s.nnz = int(col.numel())
            if ctx_handle:
                check(lib().tsg_stream_wait(ctx_handle, torch.cuda.current_stream(rp.device).cuda_stream))
            else:
                torch.cuda.current_stream(rp.device).synchronize()
        else:
            rp = np.asarray(self.rowptr)
            if rp.dtype not in (np.int32, np.int64):
                rp = rp.astype(np.int64)
            rp = np.ascontiguousarray(rp)
            col = np.ascontiguousarray(np.asarray(self.col), dtype=np.int32)
            val = np.ascontiguousarray(np.asarray(self.val), dtype=np.float64)
            keep += [rp, col, val]
            s.rowptr_bits = 64 if rp.dtype == np.int64 else 32
            s.where = _abi.MEM_HOST
            s.row_ptr = rp.ctypes.data
            s.col = col.ctypes.data if col.size else None
            s.val = val.ctypes.data if val.size else None
            s.nnz = int(col.size)
        s.owner = None
        return s, keep


def _download(ctx_handle, s: _abi.tsg_csr) -> CSR:
    rp = np.empty(s.m + 1, dtype=np.int64)
    col = np.empty(s.nnz, dtype=np.int32)
    val = np.empty(s.nnz, dtype=np.float64)
    check(lib().tsg_csr_download(ctx_handle, C.byref(s), rp.ctypes.data, col.ctypes.data if s.nnz else None,
                                 val.ctypes.data if s.nnz else None))
    return CSR(s.m, s.n, rp, col, val)


class OwnedCSR:
    """A C produced by the library (device pool memory or pinned host memory).

    Valid until ``free()`` (or garbage collection); ``download()`` copies it
    into plain numpy arrays."""

    def __init__(self, ctx: "Context", s: _abi.tsg_csr):
        self._ctx = ctx
        self.s = s

    m = property(lambda self: self.s.m)
    n = property(lambda self: self.s.n)
    nnz = property(lambda self: self.s.nnz)
    rowptr_bits = property(lambda self: self.s.rowptr_bits)
    where = property(lambda self: "device" if self.s.where == _abi.MEM_DEVICE else "host")

    def download(self) -> CSR:
        return _download(self._ctx.handle, self.s)

    def rowptr(self) -> np.ndarray:
        """The whole row pointer (int64), without the entries."""
        rp = np.empty(self.s.m + 1, dtype=np.int64)
        check(lib().tsg_csr_download_rows(self._ctx.handle, C.byref(self.s), 0, self.s.m, rp.ctypes.data,
                                          None, None))
        return rp

    def rows(self, r0: int, r1: int) -> tuple[np.ndarray, np.ndarray, np.ndarray]:
        """Rows [r0, r1): (row pointer relative to row r0, columns, values)."""
        rp = np.empty(r1 - r0 + 1, dtype=np.int64)
        lib_ = lib()
        check(lib_.tsg_csr_download_rows(self._ctx.handle, C.byref(self.s), r0, r1, rp.ctypes.data, None, None))
        cnt = int(rp[-1] - rp[0])
        col = np.empty(cnt, dtype=np.int32)
        val = np.empty(cnt, dtype=np.float64)
        if cnt:
            check(lib_.tsg_csr_download_rows(self._ctx.handle, C.byref(self.s), r0, r1, rp.ctypes.data,
                                             col.ctypes.data, val.ctypes.data))
        return rp - rp[0], col, val

    def free(self) -> None:
        if self.s.owner:
            lib().tsg_csr_free(self._ctx.handle, C.byref(self.s))

    def __del__(self):
        try:
            if self._ctx.handle:
                self.free()
        except Exception:
            pass


@dataclass
class Tiles:
    """The reference's 16x16 tile form of a matrix (host copies)."""
    m: int
    n: int
    blkm: int
    blkn: int
    blkrowptr: np.ndarray   # int64, blkm+1
    blkcolidx: np.ndarray   # int32, numblk
    nnzb: np.ndarray        # int64, numblk+1
    ptr: np.ndarray         # uint8, 16*numblk
    col: np.ndarray         # uint8, nnz (local column)
    val: np.ndarray         # float64, nnz
    mask: np.ndarray        # uint16, 16*numblk

    @property
    def numblk(self) -> int:
        return int(self.blkcolidx.shape[0])


def _download_tiles(ctx_handle, t: _abi.tsg_tiles) -> Tiles:
    nb, nnz = int(t.numblk), int(t.nnz)
    out = Tiles(t.m, t.n, t.blkm, t.blkn,
                np.empty(t.blkm + 1, np.int64), np.empty(nb, np.int32), np.empty(nb + 1, np.int64),
                np.empty(nb * 16, np.uint8), np.empty(nnz, np.uint8), np.empty(nnz, np.float64),
                np.empty(nb * 16, np.uint16))

    def p(a):
        return a.ctypes.data if a.size else None
    check(lib().tsg_tiles_download(ctx_handle, C.byref(t), p(out.blkrowptr), p(out.blkcolidx), p(out.nnzb),
                                   p(out.ptr), p(out.col), p(out.val), p(out.mask)))
    return out


class Plan:
    """The symbolic phase of op(A, B) kept on the device (tsg_plan_*): later
    products with the same patterns and new values run only the numeric step."""

    def __init__(self, ctx: "Context", A, B, op: str, batched: bool = False):
        """A plain plan of op(A, B), or with batched=True a batched plan of the
        lists A[i], B[i] (tsg_plan_create_batched)."""
        h = C.c_void_p()
        st = _abi.tsg_stats()
        if batched:
            n = len(A)
            a = (_abi.tsg_csr * n)()
            keep: list = []
            for i, X in enumerate(A):
                s_, k_ = X._tsg()
                a[i] = s_
                keep.append(k_)
            b_ptr = None
            if B is not None:
                b = (_abi.tsg_csr * n)()
                for i, X in enumerate(B):
                    s_, k_ = X._tsg()
                    b[i] = s_
                    keep.append(k_)
                b_ptr = b
            check(lib().tsg_plan_create_batched(ctx.handle, _OPS[op], n, a, b_ptr, C.byref(h), C.byref(st)))
            del keep
            self.m = self.n = None
        else:
            a, keep_a = A._tsg()
            b_ptr = None
            keep_b: list = []
            if B is not None:
                b, keep_b = B._tsg()
                b_ptr = C.byref(b)
            check(lib().tsg_plan_create(ctx.handle, _OPS[op], C.byref(a), b_ptr, C.byref(h), C.byref(st)))
            del keep_a, keep_b
            self.m, self.n = A.m, (B.n if B is not None else (A.n if op == "AA" else A.m))
        self._ctx, self.handle, self.op, self.stats = ctx, h, op, st.as_dict()

    @property
    def count(self) -> int:
        return int(lib().tsg_plan_count(self.handle))

    def value_offsets(self) -> tuple[np.ndarray, np.ndarray]:
        """Where each instance's values start in set_values' arrays (count+1 each)."""
        n = self.count
        ao = np.zeros(n + 1, np.int64)
        bo = np.zeros(n + 1, np.int64)
        check(lib().tsg_plan_value_offsets(self.handle, ao.ctypes.data, bo.ctypes.data))
        return ao, bo

    def set_values(self, valA, valB=None) -> None:
        """New values (host numpy) for the resident numeric step."""
        a = np.ascontiguousarray(np.asarray(valA), dtype=np.float64)
        b = None if valB is None else np.ascontiguousarray(np.asarray(valB), dtype=np.float64)
        check(lib().tsg_plan_set_values(self._ctx.handle, self.handle, a.ctypes.data if a.size else None,
                                        (b.ctypes.data if b.size else None) if b is not None else None, _abi.MEM_HOST))

    def replay(self) -> None:
        """Numeric step on the resident values as one CUDA graph (asynchronous)."""
        check(lib().tsg_plan_replay(self._ctx.handle, self.handle))

    def tune(self) -> float:
        """Pick the fastest numeric variant and bin thresholds for this plan;
        returns its time in ms."""
        ms = C.c_double()
        check(lib().tsg_plan_tune(self._ctx.handle, self.handle, C.byref(ms)))
        return ms.value

    def settings(self) -> dict:
        """Numeric settings and bin thresholds the plan runs with."""
        v = [C.c_int32() for _ in range(5)]
        check(lib().tsg_plan_settings(self.handle, *[C.byref(x) for x in v]))
        return dict(zip(("threads", "walk", "dense_tile_min", "smem_acc_max", "row_acc_max"), (x.value for x in v)))

    def result(self, instance: int = 0) -> CSR:
        """Host copy of instance `instance` of the resident C (after replay)."""
        c = _abi.tsg_csr()
        check(lib().tsg_plan_result(self._ctx.handle, self.handle, int(instance), C.byref(c)))
        return _download(self._ctx.handle, c)

    @property
    def nnz(self) -> int:
        return int(lib().tsg_plan_nnz(self.handle))

    @property
    def device_bytes(self) -> int:
        return int(lib().tsg_plan_device_bytes(self.handle))

    def execute_raw(self, valA, valB=None, out: str = "host", stats: bool = False):
        """C with new values (numpy arrays on the host, or torch CUDA tensors)."""
        keep = []

        def ptr(v):
            if v is None:
                return None, _abi.MEM_HOST
            if hasattr(v, "is_cuda") and v.is_cuda:
                import torch
                v = v.contiguous()
                keep.append(v)
                torch.cuda.current_stream(v.device).synchronize()
                return v.data_ptr(), _abi.MEM_DEVICE
            a = np.ascontiguousarray(np.asarray(v), dtype=np.float64)
            keep.append(a)
            return (a.ctypes.data if a.size else None), _abi.MEM_HOST
        pa, wa = ptr(valA)
        pb, wb = ptr(valB)
        where = wa if valA is not None else wb
        if valB is not None and wb != where:
            raise ValueError("valA and valB must both be host or both be device arrays")
        c = _abi.tsg_csr()
        c.where = _abi.MEM_DEVICE if out == "device" else _abi.MEM_HOST
        st = _abi.tsg_stats() if stats else None
        check(lib().tsg_plan_execute(self._ctx.handle, self.handle, pa, pb, where, C.byref(c),
                                     C.byref(st) if st is not None else None))
        del keep
        return OwnedCSR(self._ctx, c), (st.as_dict() if st is not None else None)

    def execute(self, valA, valB=None) -> CSR:
        oc, _ = self.execute_raw(valA, valB, out="host")
        res = oc.download()
        oc.free()
        return res

    def close(self) -> None:
        if self.handle:
            lib().tsg_plan_destroy(self._ctx.handle, self.handle)
            self.handle = None

    def __del__(self):
        try:
            if self._ctx.handle:
                self.close()
        except Exception:
            pass


class Context:
    """One device, one stream, one memory pool (tsg_create / tsg_destroy)."""

    def __init__(self, device: int = 0, **opts):
        o = _abi.tsg_opts()
        lib().tsg_opts_default(C.byref(o))
        for k, v in opts.items():
            if not hasattr(o, k):
                raise TypeError(f"unknown option {k}")
            setattr(o, k, int(v))
        self.opts = o
        h = C.c_void_p()
        check(lib().tsg_create(C.byref(h), int(device), C.byref(o)))
        self.handle = h
        self.device = device

    def close(self) -> None:
        if self.handle:
            lib().tsg_destroy(self.handle)
            self.handle = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def spgemm_raw(self, A: CSR, B: CSR | None = None, op: str = "AA", out: str = "host",
                   stats: bool = False) -> tuple[OwnedCSR, dict | None]:
        """C = op(A, B) left in library-owned memory (`out` = "host" pinned or "device")."""
        a, keep_a = A._tsg(self.handle)
        b_ptr = None
        keep_b: list = []
        if B is not None:
            b, keep_b = B._tsg(self.handle)
            b_ptr = C.byref(b)
        c = _abi.tsg_csr()
        c.where = _abi.MEM_DEVICE if out == "device" else _abi.MEM_HOST
        st = _abi.tsg_stats() if stats else None
        check(lib().tsg_spgemm(self.handle, _OPS[op], C.byref(a), b_ptr, C.byref(c),
                               C.byref(st) if st is not None else None))
        del keep_a, keep_b
        return OwnedCSR(self, c), (st.as_dict() if st is not None else None)

    def load_mtx_device(self, path: str) -> tuple[OwnedCSR, bool]:
        """Matrix Market file -> device CSR, the data lines parsed on the GPU
        (tsg_load_mtx_device; the same matrix as load_mtx)."""
        s = _abi.tsg_csr()
        sym = C.c_int32(0)
        check(lib().tsg_load_mtx_device(self.handle, str(path).encode(), C.byref(s), C.byref(sym)))
        return OwnedCSR(self, s), bool(sym.value)

    def spgemm(self, A: CSR, B: CSR | None = None, op: str = "AA", stats: bool = False):
        """C = op(A, B) as a host CSR (numpy).  op: "AA", "AAT" or "AB"."""
        oc, st = self.spgemm_raw(A, B, op, out="host", stats=stats)
        res = oc.download()
        oc.free()
        return (res, st) if stats else res

    def spgemm_batched_raw(self, As: list, Bs: list | None = None, op: str = "AA", out: str = "host",
                           stats: bool = False):
        """C_i = op(A_i, B_i) for all instances in one pipeline pass (tsg_spgemm_batched);
        returns OwnedCSR views that share one allocation."""
        n = len(As)
        a = (_abi.tsg_csr * max(n, 1))()
        keep: list = []
        for i, A in enumerate(As):
            s_, k_ = A._tsg()
            a[i] = s_
            keep.append(k_)
        b_ptr = None
        if Bs is not None:
            b = (_abi.tsg_csr * max(n, 1))()
            for i, B in enumerate(Bs):
                s_, k_ = B._tsg()
                b[i] = s_
                keep.append(k_)
            b_ptr = b
        c = (_abi.tsg_csr * max(n, 1))()
        c[0].where = _abi.MEM_DEVICE if out == "device" else _abi.MEM_HOST
        st = _abi.tsg_stats() if stats else None
        check(lib().tsg_spgemm_batched(self.handle, _OPS[op], n, a, b_ptr, c, C.byref(st) if st is not None else None))
        del keep
        outs = []
        for i in range(n):
            cs = _abi.tsg_csr()
            C.memmove(C.byref(cs), C.byref(c[i]), C.sizeof(_abi.tsg_csr))
            outs.append(OwnedCSR(self, cs))
        return outs, (st.as_dict() if st is not None else None)

    def spgemm_batched(self, As: list, Bs: list | None = None, op: str = "AA") -> list:
        """Host CSRs C_i = op(A_i, B_i), computed as one batched SpGEMM."""
        outs, _ = self.spgemm_batched_raw(As, Bs, op, out="host")
        res = [o.download() for o in outs]
        for o in outs:
            o.free()
        return res

    def plan(self, A: CSR, B: CSR | None = None, op: str = "AA") -> Plan:
        """Symbolic phase of op(A, B), kept for numeric-only repeats."""
        return Plan(self, A, B, op)

    def plan_batched(self, As: list, Bs: list | None = None, op: str = "AA") -> Plan:
        """Symbolic phase of op(A_i, B_i) for all instances, packed (tsg_plan_create_batched)."""
        return Plan(self, As, Bs, op, batched=True)

    def spgemm_tiles(self, A: CSR, B: CSR | None = None, op: str = "AA") -> Tiles:
        """C = op(A, B) in the reference's tile form (tsg_spgemm_tiles)."""
        a, keep_a = A._tsg()
        b_ptr = None
        keep_b: list = []
        if B is not None:
            b, keep_b = B._tsg()
            b_ptr = C.byref(b)
        t = _abi.tsg_tiles()
        check(lib().tsg_spgemm_tiles(self.handle, _OPS[op], C.byref(a), b_ptr, C.byref(t), None))
        try:
            return _download_tiles(self.handle, t)
        finally:
            lib().tsg_tiles_free(self.handle, C.byref(t))
            del keep_a, keep_b

    def csr_to_tiles(self, A: CSR) -> Tiles:
        a, keep = A._tsg()
        t = _abi.tsg_tiles()
        check(lib().tsg_csr_to_tiles(self.handle, C.byref(a), C.byref(t)))
        try:
            return _download_tiles(self.handle, t)
        finally:
            lib().tsg_tiles_free(self.handle, C.byref(t))
            del keep

    def tiles_roundtrip(self, A: CSR) -> CSR:
        """CSR -> tiles -> CSR entirely on the device (tsg_csr_to_tiles + tsg_tiles_to_csr)."""
        a, keep = A._tsg()
        t = _abi.tsg_tiles()
        check(lib().tsg_csr_to_tiles(self.handle, C.byref(a), C.byref(t)))
        c = _abi.tsg_csr()
        try:
            check(lib().tsg_tiles_to_csr(self.handle, C.byref(t), C.byref(c)))
            res = _download(self.handle, c)
            lib().tsg_csr_free(self.handle, C.byref(c))
            return res
        finally:
            lib().tsg_tiles_free(self.handle, C.byref(t))
            del keep


def load_mtx(path: str) -> tuple[CSR, bool]:
    """Matrix Market file -> host CSR with mmio_allinone semantics; returns (A, is_symmetric)."""
    s = _abi.tsg_csr()
    sym = C.c_int32(0)
    check(lib().tsg_load_mtx(str(path).encode(), C.byref(s), C.byref(sym)))
    try:
        out = _download(None, s)
        out.rowptr = out.rowptr.astype(np.int32)
        return out, bool(sym.value)
    finally:
        lib().tsg_csr_free(None, C.byref(s))


def write_mtx(path: str, A: CSR, exact: bool = False) -> None:
    """Host CSR -> Matrix Market coordinate file in the reference's writer
    format (mm_write_mtx_crd); exact=True keeps every bit of the values."""
    if A.on_device:
        raise ValueError("write_mtx takes a host matrix")
    a, keep = A._tsg()
    check(lib().tsg_write_mtx(str(path).encode(), C.byref(a), int(bool(exact))))
    del keep


def version() -> str:
    return lib().tsg_version().decode()


def pinned_cache_cap() -> int:
    """Bytes of pinned host memory kept for reuse by host results
    (TSG_PINNED_CACHE_BYTES, else min(96 GB, 3/8 of host memory))."""
    return int(lib().tsg_pinned_cache_cap())


__all__ = ["CSR", "Context", "OwnedCSR", "Plan", "Tiles", "TSGError", "load_mtx", "write_mtx", "version",
           "pinned_cache_cap"]
