"""Generate the golden fixtures in tests/golden/ from the reference's own code.

Run where the reference checkout is present (it builds oracle/_ref first):

    python tests/golden/make_golden.py

Sources of truth, all compiled unmodified from the reference by
oracle/build_ref.sh:
  * thmkl_dcsrmultcsr   thmkl_dcsrmultcsr.c:7-95 -- C = A*B in CSR (the reference CPU path)
  * matrix_transposition utils.h:158-195       -- B = A^T for the A*A^T cases
  * blocknnz/blkmessage  main_spgemm-col.cu:44-120 (+ quick_sort_key, utils.h) -- A's tile structure
  * step1/step2          main_spgemm-col.cu:122-188, :572-627 -- C's tile structure
  * step3/step4          main_spgemm-col.cu:899-994, :4073-4179 -- C's tile nnz, row starts,
                         local columns and values
  * mmio_allinone        mmio_highlevel.h:593-759 -- the Matrix Market load path
step3/step4 consume A in tile-CSR and B in tile-CSC; those payloads come
from the oracle's restatement of the host conversion (main_spgemm-col.cu:
4968-5351), so the fixtures pin that conversion end to end: a wrong payload
would make the reference's step4 disagree with thmkl_dcsrmultcsr.

Each case is written as <name>.npz (inputs and reference outputs); the
mtx/*.mtx files are small hand-written inputs whose reference loads are
stored as mtx_<name>.npz.
"""
from __future__ import annotations

import ctypes as C
import subprocess
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parents[1]
sys.path.insert(0, str(ROOT))

from oracle import oracle as O  # noqa: E402
from tilespgemm_gb300 import matrices as M  # noqa: E402
from tilespgemm_gb300.api import CSR  # noqa: E402

REF = ROOT / "oracle" / "_ref"
IP = C.POINTER(C.c_int)
DP = C.POINTER(C.c_double)


def _load_ref():
    subprocess.run(["bash", str(ROOT / "oracle" / "build_ref.sh")], check=True)
    th = C.CDLL(str(REF / "libthmkl_ref.so"))
    st = C.CDLL(str(REF / "libstir_ref.so"))
    return th, st


def p(a):
    return a.ctypes.data_as(C.c_void_p)


def ref_thmkl(th, A: CSR, B: CSR):
    m, n, k = C.c_int(A.m), C.c_int(A.n), C.c_int(B.n)
    ia = np.ascontiguousarray(A.rowptr, np.int32); ja = np.ascontiguousarray(A.col, np.int32)
    a = np.ascontiguousarray(A.val, np.float64)
    ib = np.ascontiguousarray(B.rowptr, np.int32); jb = np.ascontiguousarray(B.col, np.int32)
    b = np.ascontiguousarray(B.val, np.float64)
    ic = np.zeros(A.m + 1, np.int32)
    req, srt, nz, info = C.c_int(1), C.c_int(1), C.c_int(0), C.c_int(0)
    dummy_c = np.zeros(1, np.float64); dummy_j = np.zeros(1, np.int32)
    f = th.thmkl_dcsrmultcsr
    f.restype = None
    f(b"n", C.byref(req), C.byref(srt), C.byref(m), C.byref(n), C.byref(k), p(a), p(ja), p(ia), p(b), p(jb), p(ib),
      p(dummy_c), p(dummy_j), p(ic), C.byref(nz), C.byref(info))
    nnz = int(ic[-1])
    jc = np.zeros(max(nnz, 1), np.int32); c = np.zeros(max(nnz, 1), np.float64)
    req = C.c_int(0)
    f(b"n", C.byref(req), C.byref(srt), C.byref(m), C.byref(n), C.byref(k), p(a), p(ja), p(ia), p(b), p(jb), p(ib),
      p(c), p(jc), p(ic), C.byref(nz), C.byref(info))
    return ic, jc[:nnz], c[:nnz]


def ref_transpose(st, A: CSR) -> CSR:
    rp = np.ascontiguousarray(A.rowptr, np.int32); col = np.ascontiguousarray(A.col, np.int32)
    val = np.ascontiguousarray(A.val, np.float64)
    trow = np.zeros(max(A.nnz, 1), np.int32); tp = np.zeros(A.n + 1, np.int32)
    tv = np.zeros(max(A.nnz, 1), np.float64)
    st.ref_matrix_transposition(A.m, A.n, A.nnz, p(rp), p(col), p(val), p(trow), p(tp), p(tv))
    return CSR(A.n, A.m, tp.astype(np.int64), trow[:A.nnz], tv[:A.nnz])


def ref_tile_structure(st, A: CSR):
    rp = np.ascontiguousarray(A.rowptr, np.int32); col = np.ascontiguousarray(A.col, np.int32)
    rb, cb, nb = C.c_int(0), C.c_int(0), C.c_int(0)
    st.ref_blocknnz(C.byref(rb), C.byref(cb), p(col), p(rp), A.m, A.n, C.byref(nb))
    brp = np.zeros(rb.value + 1, np.int32); bci = np.zeros(max(nb.value, 1), np.int32)
    st.ref_blkmessage(C.byref(rb), C.byref(cb), p(col), p(rp), A.m, A.n, p(brp), p(bci))
    for i in range(rb.value):
        seg = bci[brp[i]:brp[i + 1]]
        if seg.size > 1:
            tmp = np.ascontiguousarray(seg)
            st.ref_quick_sort_key(p(tmp), tmp.size)
            bci[brp[i]:brp[i + 1]] = tmp
    return brp, bci[:nb.value]


def ref_steps(st, A: CSR, B: CSR):
    ta, tb, tbr = O.tile_csr(A), O.tile_csc(B), O.tile_csr(B)
    blkmA, blknA = ta["blkm"], ta["blkn"]
    blkmB, blknB = tb["blkm"], tb["blkn"]
    arp = np.ascontiguousarray(ta["blkrowptr"], np.int32); aci = np.ascontiguousarray(ta["blkcolidx"], np.int32)
    bcp = np.ascontiguousarray(tb["blkcolptr"], np.int32); bri = np.ascontiguousarray(tb["blkrowidx"], np.int32)
    crp = np.zeros(blkmA + 1, np.int32)
    nbc = C.c_int(0)
    st.ref_step1(p(arp), p(aci), blkmA, blknA, p(bcp), p(bri), blkmB, blknB, p(crp), C.byref(nbc))
    cci = np.zeros(max(nbc.value, 1), np.int32)
    st.ref_step2(p(arp), p(aci), blkmA, blknA, p(bcp), p(bri), blkmB, blknB, p(crp), p(cci))
    nnzbA = np.ascontiguousarray(ta["nnzb"], np.int32)
    valA = np.ascontiguousarray(ta["val"] if A.nnz else np.zeros(1), np.float64)
    colA = np.ascontiguousarray(ta["lcol"] if A.nnz else np.zeros(1, np.uint8), np.uint8)
    ptrA = np.ascontiguousarray(ta["ptr"] if ta["numblk"] else np.zeros(16, np.uint8), np.uint8)
    nnzbB = np.ascontiguousarray(tb["nnzb"], np.int32)
    valB = np.ascontiguousarray(tb["val"] if B.nnz else np.zeros(1), np.float64)
    colB = np.ascontiguousarray(tb["lcol"] if B.nnz else np.zeros(1, np.uint8), np.uint8)
    ptrB = np.ascontiguousarray(tb["ptr"] if tb["numblk"] else np.zeros(16, np.uint8), np.uint8)
    nnzbC = np.zeros(nbc.value + 1, np.int32)
    nnzC = C.c_int(0)
    common = [p(arp), p(aci), blkmA, blknA, p(nnzbA), A.m, p(valA), p(colA), p(ptrA),
              p(bcp), p(bri), blkmB, blknB, p(nnzbB), p(valB), p(colB), p(ptrB), p(crp), p(cci)]
    st.ref_step3(*common, p(nnzbC), C.byref(nnzC))
    valC = np.zeros(max(nnzC.value, 1), np.float64)
    colC = np.zeros(max(nnzC.value, 1), np.uint8)
    ptrC = np.zeros(max(nbc.value * 16, 16), np.uint8)
    st.ref_step4(*common, p(nnzbC), p(valC), p(colC), p(ptrC))
    return dict(blkrowptrC=crp, blkcolidxC=cci[:nbc.value], nnzbC=nnzbC, ptrC=ptrC[:nbc.value * 16],
                colC=colC[:nnzC.value], valC=valC[:nnzC.value], tile_blkrowptrB=tbr["blkrowptr"],
                tile_blkcolidxB=tbr["blkcolidx"])


def cases():
    out = {}
    out["lap16_AA"] = (M.laplacian_2d(16), "AA")
    out["lap13x11_AA_refval"] = (M.ref_values(M.laplacian_2d(13, 11)), "AA")
    out["rand100_AA"] = (M.random_sparse(100, 100, 5, seed=3), "AA")
    out["rand100_AA_refval"] = (M.ref_values(M.random_sparse(100, 100, 5, seed=3)), "AA")
    out["band300_AA"] = (M.random_sparse(300, 300, 7, seed=4, band=20), "AA")
    out["rect77x130_AAT"] = (M.random_sparse(77, 130, 6, seed=5), "AAT")
    out["rect77x130_AAT_refval"] = (M.ref_values(M.random_sparse(77, 130, 6, seed=5)), "AAT")
    out["rmat8_AAT"] = (M.rmat(8, 8, seed=2), "AAT")
    out["st27_5_AA"] = (M.stencil_27(5, seed=1), "AA")
    out["dup_unsorted64_AA"] = (M.random_sparse(64, 64, 6, seed=7, dup=True, unsorted=True), "AA")
    out["dup_unsorted64_AA_refval"] = (M.ref_values(M.random_sparse(64, 64, 6, seed=7, dup=True, unsorted=True)), "AA")
    out["emptyrows90_AA"] = (M.random_sparse(90, 90, 4, seed=8, empty_rows=0.3), "AA")
    out["tiny5_AA"] = (M.random_sparse(5, 5, 2, seed=9), "AA")
    out["wide40x3000_AAT"] = (M.random_sparse(40, 3000, 30, seed=10), "AAT")
    return out


def main() -> None:
    th, st = _load_ref()
    for name, (A, op) in cases().items():
        A = CSR(A.m, A.n, np.asarray(A.rowptr, np.int64), np.asarray(A.col, np.int32), np.asarray(A.val, np.float64))
        B = A if op == "AA" else ref_transpose(st, A)
        ic, jc, c = ref_thmkl(th, A, B)
        brpA, bciA = ref_tile_structure(st, A)
        steps = ref_steps(st, A, B)
        np.savez_compressed(HERE / f"{name}.npz", m=A.m, n=A.n, op=op,
                            a_rowptr=A.rowptr, a_col=A.col, a_val=A.val,
                            b_rowptr=B.rowptr, b_col=B.col, b_val=B.val,
                            c_rowptr=ic.astype(np.int64), c_col=jc, c_val=c,
                            a_blkrowptr=brpA, a_blkcolidx=bciA, **steps)
        print(f"{name}: m={A.m} n={A.n} nnzA={A.nnz} nnzC={int(ic[-1])} tilesC={steps['blkcolidxC'].size}")
    # Matrix Market loads
    for f in sorted((HERE / "mtx").glob("*.mtx")):
        m, n, nnz, sym = C.c_int(0), C.c_int(0), C.c_int(0), C.c_int(0)
        rp, col, val = IP(), IP(), DP()
        rc = st.ref_mmio_allinone(C.byref(m), C.byref(n), C.byref(nnz), C.byref(sym), C.byref(rp), C.byref(col),
                                  C.byref(val), str(f).encode())
        if rc != 0:
            np.savez_compressed(HERE / f"mtx_{f.stem}.npz", rc=rc)
            print(f"mtx {f.name}: reference loader returns {rc}")
            continue
        rpa = np.array([rp[i] for i in range(m.value + 1)], np.int32)
        cola = np.array([col[i] for i in range(nnz.value)], np.int32)
        vala = np.array([val[i] for i in range(nnz.value)], np.float64)
        np.savez_compressed(HERE / f"mtx_{f.stem}.npz", rc=0, m=m.value, n=n.value, nnz=nnz.value, sym=sym.value,
                            rowptr=rpa, col=cola, val=vala)
        print(f"mtx {f.name}: {m.value}x{n.value} nnz={nnz.value} sym={sym.value}")


if __name__ == "__main__":
    main()
