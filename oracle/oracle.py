"""ctypes wrapper of the CPU oracle (oracle/tsg_oracle.c).

TEST INFRASTRUCTURE ONLY: used by tests/, __graft_entry__.smoke() and the
CPU-baseline leg of bench.py as the checker.  The library never imports it.
Every function here calls the C restatement; the reference file:line each
one follows is documented in tsg_oracle.c.
"""
from __future__ import annotations

import ctypes as C
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB_PATH = HERE / "liboracle.so"
_lib = None

P = C.c_void_p


def _build() -> None:
    subprocess.run(["gcc", "-O3", "-fopenmp", "-ffp-contract=off", "-fPIC", "-shared", "-Wall",
                    str(HERE / "tsg_oracle.c"), "-o", str(LIB_PATH), "-lm"], check=True)


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        src = HERE / "tsg_oracle.c"
        if not LIB_PATH.exists() or LIB_PATH.stat().st_mtime < src.stat().st_mtime:
            _build()
        L = C.CDLL(str(LIB_PATH))
        L.orc_spgemm_rownnz.restype = C.c_int
        L.orc_spgemm_rownnz.argtypes = [C.c_int, C.c_int, P, P, P, P, P]
        L.orc_spgemm_fill.restype = C.c_int
        L.orc_spgemm_fill.argtypes = [C.c_int, C.c_int, P, P, P, P, P, P, P, P, P, P]
        L.orc_spgemm_rows.restype = C.c_int
        L.orc_spgemm_rows.argtypes = [C.c_int, P, C.c_int, C.c_int, P, P, P, P, P, P, P, P, P, P]
        L.orc_thmkl_rows.restype = None
        L.orc_thmkl_rows.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int, P, P, P, P, P, P, P, P, P]
        L.orc_transpose.restype = None
        L.orc_transpose.argtypes = [C.c_int, C.c_int, P, P, P, P, P, P]
        L.orc_tile_rowptr.restype = C.c_int64
        L.orc_tile_rowptr.argtypes = [C.c_int, C.c_int, P, P, P]
        L.orc_tile_fill.restype = None
        L.orc_tile_fill.argtypes = [C.c_int, C.c_int, P, P, P, P, P, P, P, P, P, P, P]
        L.orc_tile_csc_fill.restype = None
        L.orc_tile_csc_fill.argtypes = [C.c_int, C.c_int, P, P, P, P, P, P, P, P, P, P]
        L.orc_tile_symbolic.restype = C.c_int64
        L.orc_tile_symbolic.argtypes = [C.c_int, P, P, C.c_int, P, P, P, P]
        L.orc_tile_numeric.restype = C.c_int64
        L.orc_tile_numeric.argtypes = [C.c_int, C.c_int, P, P, P, P, P, P, P, P, P, P, P, P, P, P, P, P, P, P, P]
        L.orc_tiles_to_csr.restype = None
        L.orc_tiles_to_csr.argtypes = [C.c_int, C.c_int, P, P, P, P, P, P, P, P, P]
        L.orc_nnzcub.restype = C.c_int64
        L.orc_nnzcub.argtypes = [C.c_int, P, P, P]
        L.orc_max_threads.restype = C.c_int
        L.orc_set_threads.argtypes = [C.c_int]
        _lib = L
    return _lib


def _p(a: np.ndarray | None):
    return None if a is None else a.ctypes.data


def _csr64(A):
    rp = np.ascontiguousarray(np.asarray(A.rowptr), dtype=np.int64)
    col = np.ascontiguousarray(np.asarray(A.col), dtype=np.int32)
    val = np.ascontiguousarray(np.asarray(A.val), dtype=np.float64)
    return rp, col, val


def spgemm(A, B, with_bound: bool = False):
    """C = A*B (CSR, int64 row pointer) in the reference CPU order with FMA rounding.
    Returns (rowptr, col, val) or (rowptr, col, val, bound)."""
    L = lib()
    arp, acol, aval = _csr64(A)
    brp, bcol, bval = _csr64(B)
    m, n = int(A.m), int(B.n)
    crp = np.zeros(m + 1, dtype=np.int64)
    if L.orc_spgemm_rownnz(m, n, _p(arp), _p(acol), _p(brp), _p(bcol), _p(crp)) != 0:
        raise ValueError("column index out of range")
    nnz = int(crp[-1])
    ccol = np.empty(max(nnz, 1), dtype=np.int32)
    cval = np.empty(max(nnz, 1), dtype=np.float64)
    bnd = np.empty(max(nnz, 1), dtype=np.float64) if with_bound else None
    L.orc_spgemm_fill(m, n, _p(arp), _p(acol), _p(aval), _p(brp), _p(bcol), _p(bval), _p(crp),
                      _p(ccol), _p(cval), _p(bnd))
    out = (crp, ccol[:nnz], cval[:nnz])
    return out + (bnd[:nnz],) if with_bound else out


def spgemm_rows(A, B, rows):
    """Rows `rows` (any order, no repeats needed) of C = A*B, as spgemm()
    computes them: (rowptr relative to the list, col, val, bound), the
    bound being sum |a||b| per entry."""
    L = lib()
    arp, acol, aval = _csr64(A)
    brp, bcol, bval = _csr64(B)
    rows = np.ascontiguousarray(np.asarray(rows), dtype=np.int32)
    nr = len(rows)
    crp = np.zeros(nr + 1, dtype=np.int64)
    if L.orc_spgemm_rows(nr, _p(rows), int(A.m), int(B.n), _p(arp), _p(acol), None, _p(brp), _p(bcol), None,
                         _p(crp), None, None, None) != 0:
        raise ValueError("row or column index out of range")
    nnz = int(crp[-1])
    ccol = np.empty(max(nnz, 1), dtype=np.int32)
    cval = np.empty(max(nnz, 1), dtype=np.float64)
    bnd = np.empty(max(nnz, 1), dtype=np.float64)
    L.orc_spgemm_rows(nr, _p(rows), int(A.m), int(B.n), _p(arp), _p(acol), _p(aval), _p(brp), _p(bcol),
                      _p(bval), _p(crp), _p(ccol), _p(cval), _p(bnd))
    return crp, ccol[:nnz], cval[:nnz], bnd[:nnz]


def transpose(A):
    """Stable CSR transpose (utils.h:158-195): (rowptr int64, col, val) of A^T."""
    L = lib()
    rp, col, val = _csr64(A)
    tp = np.zeros(A.n + 1, dtype=np.int64)
    tr = np.empty(max(A.nnz, 1), dtype=np.int32)
    tv = np.empty(max(A.nnz, 1), dtype=np.float64)
    L.orc_transpose(A.m, A.n, _p(rp), _p(col), _p(val), _p(tp), _p(tr), _p(tv))
    return tp, tr[:A.nnz], tv[:A.nnz]


def nnzcub(A, B) -> int:
    arp, acol, _ = _csr64(A)
    brp, _, _ = _csr64(B)
    return int(lib().orc_nnzcub(A.m, _p(arp), _p(acol), _p(brp)))


def tile_csr(A) -> dict:
    """A in the reference's tile-CSR form (main_spgemm-col.cu:4968-5240)."""
    L = lib()
    rp, col, val = _csr64(A)
    blkm = (A.m + 15) // 16
    trp = np.zeros(blkm + 1, dtype=np.int32)
    nb = int(L.orc_tile_rowptr(A.m, A.n, _p(rp), _p(col), _p(trp)))
    t = dict(blkm=blkm, blkn=(A.n + 15) // 16, blkrowptr=trp,
             blkcolidx=np.zeros(max(nb, 1), np.int32), nnzb=np.zeros(nb + 1, np.int32),
             ptr=np.zeros(max(nb * 16, 1), np.uint8), idx=np.zeros(max(A.nnz, 1), np.uint8),
             lcol=np.zeros(max(A.nnz, 1), np.uint8), val=np.zeros(max(A.nnz, 1), np.float64),
             mask=np.zeros(max(nb * 16, 1), np.uint16))
    L.orc_tile_fill(A.m, A.n, _p(rp), _p(col), _p(val), _p(trp), _p(t["blkcolidx"]), _p(t["nnzb"]),
                    _p(t["ptr"]), _p(t["idx"]), _p(t["lcol"]), _p(t["val"]), _p(t["mask"]))
    for k, ln in (("blkcolidx", nb), ("ptr", nb * 16), ("mask", nb * 16), ("idx", A.nnz),
                  ("lcol", A.nnz), ("val", A.nnz)):
        t[k] = t[k][:ln]
    t["numblk"] = nb
    return t


def tile_csc(B) -> dict:
    """B in the reference's tile-CSC form (main_spgemm-col.cu:5003-5351)."""
    L = lib()
    kB, nB = int(B.m), int(B.n)
    tp, tr, tv = transpose(B)
    blkn = (nB + 15) // 16
    cp = np.zeros(blkn + 1, dtype=np.int32)
    nb = int(L.orc_tile_rowptr(nB, kB, _p(tp), _p(tr), _p(cp)))
    t = dict(blkm=(kB + 15) // 16, blkn=blkn, blkcolptr=cp, blkrowidx=np.zeros(max(nb, 1), np.int32),
             nnzb=np.zeros(nb + 1, np.int32), ptr=np.zeros(max(nb * 16, 1), np.uint8),
             lcol=np.zeros(max(B.nnz, 1), np.uint8), val=np.zeros(max(B.nnz, 1), np.float64),
             mask=np.zeros(max(nb * 16, 1), np.uint16))
    L.orc_tile_csc_fill(kB, nB, _p(tp), _p(tr), _p(tv), _p(cp), _p(t["blkrowidx"]), _p(t["nnzb"]),
                        _p(t["ptr"]), _p(t["lcol"]), _p(t["val"]), _p(t["mask"]))
    for k, ln in (("blkrowidx", nb), ("ptr", nb * 16), ("mask", nb * 16), ("lcol", B.nnz), ("val", B.nnz)):
        t[k] = t[k][:ln]
    t["numblk"] = nb
    return t


def tile_spgemm(A, B) -> dict:
    """C = A*B in tile form (structure per step1/step2, nnz/masks per step3,
    payload per step4 of main_spgemm-col.cu)."""
    L = lib()
    ta, tbr, tbc = tile_csr(A), tile_csr(B), tile_csc(B)
    blkm = ta["blkm"]
    crp = np.zeros(blkm + 1, dtype=np.int64)
    nbc = int(L.orc_tile_symbolic(blkm, _p(ta["blkrowptr"]), _p(ta["blkcolidx"]), tbr["blkn"],
                                  _p(tbr["blkrowptr"]), _p(tbr["blkcolidx"]), _p(crp), None))
    ccol = np.zeros(max(nbc, 1), np.int32)
    L.orc_tile_symbolic(blkm, _p(ta["blkrowptr"]), _p(ta["blkcolidx"]), tbr["blkn"], _p(tbr["blkrowptr"]),
                        _p(tbr["blkcolidx"]), _p(crp), _p(ccol))
    nnzb = np.zeros(nbc + 1, np.int64)
    mask = np.zeros(max(nbc * 16, 1), np.uint16)
    ptr = np.zeros(max(nbc * 16, 1), np.uint8)
    args = [A.m, blkm, _p(ta["blkrowptr"]), _p(ta["blkcolidx"]), _p(ta["nnzb"]), _p(ta["ptr"]), _p(ta["lcol"]),
            _p(ta["val"]), _p(tbc["blkcolptr"]), _p(tbc["blkrowidx"]), _p(tbc["nnzb"]), _p(tbc["ptr"]),
            _p(tbc["lcol"]), _p(tbc["val"]), _p(crp), _p(ccol), _p(nnzb), _p(mask), _p(ptr)]
    nnz = int(L.orc_tile_numeric(*args, None, None))
    col = np.zeros(max(nnz, 1), np.uint8)
    val = np.zeros(max(nnz, 1), np.float64)
    L.orc_tile_numeric(*args, _p(col), _p(val))
    return dict(blkm=blkm, blkn=tbr["blkn"], blkrowptr=crp, blkcolidx=ccol[:nbc], nnzb=nnzb,
                mask=mask[:nbc * 16], ptr=ptr[:nbc * 16], col=col[:nnz], val=val[:nnz], numblk=nbc, nnz=nnz)


def tiles_to_csr(m: int, t: dict):
    """Tile form -> CSR (rowptr int64, col, val)."""
    L = lib()
    blkm = (m + 15) // 16
    nnz = int(t["nnzb"][-1])
    crp = np.zeros(m + 1, np.int64)
    ccol = np.zeros(max(nnz, 1), np.int32)
    cval = np.zeros(max(nnz, 1), np.float64)
    brp = np.ascontiguousarray(t["blkrowptr"], dtype=np.int64)
    nnzb = np.ascontiguousarray(t["nnzb"], dtype=np.int64)
    L.orc_tiles_to_csr(m, blkm, _p(brp), _p(np.ascontiguousarray(t["blkcolidx"], np.int32)), _p(nnzb),
                       _p(np.ascontiguousarray(t["ptr"], np.uint8)), _p(np.ascontiguousarray(t["col"], np.uint8)),
                       _p(np.ascontiguousarray(t["val"], np.float64)), _p(crp), _p(ccol), _p(cval))
    return crp, ccol[:nnz], cval[:nnz]


def thmkl_rows(A, B, r0: int, r1: int):
    """Time-faithful restatement of the reference's OpenMP CPU SpGEMM
    (thmkl_dcsrmultcsr.c:7-95) on rows [r0, r1): both phases.
    Returns (rowptr relative to r0, col, val)."""
    L = lib()
    ia = np.ascontiguousarray(np.asarray(A.rowptr), dtype=np.int32)
    ja = np.ascontiguousarray(np.asarray(A.col), dtype=np.int32)
    a = np.ascontiguousarray(np.asarray(A.val), dtype=np.float64)
    ib = np.ascontiguousarray(np.asarray(B.rowptr), dtype=np.int32)
    jb = np.ascontiguousarray(np.asarray(B.col), dtype=np.int32)
    b = np.ascontiguousarray(np.asarray(B.val), dtype=np.float64)
    ic = np.zeros(r1 - r0 + 1, dtype=np.int32)
    L.orc_thmkl_rows(1, r0, r1, int(B.n), _p(a), _p(ja), _p(ia), _p(b), _p(jb), _p(ib), None, None, _p(ic))
    nnz = int(ic[-1])
    jc = np.zeros(max(nnz, 1), np.int32)
    c = np.zeros(max(nnz, 1), np.float64)
    L.orc_thmkl_rows(0, r0, r1, int(B.n), _p(a), _p(ja), _p(ia), _p(b), _p(jb), _p(ib), _p(c), _p(jc), _p(ic))
    return ic, jc[:nnz], c[:nnz]


def max_threads() -> int:
    return int(lib().orc_max_threads())


def set_threads(t: int) -> None:
    lib().orc_set_threads(int(t))
