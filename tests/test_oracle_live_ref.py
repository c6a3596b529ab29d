"""The oracle against the reference's own code, called live on seeded inputs
beyond the committed fixtures.

Where the reference's CPU code has been built into oracle/_ref (by
oracle/build_ref.sh, from a reference checkout on this machine), every
case below is computed both by the oracle and by the reference:
- the CSR product (thmkl_dcsrmultcsr.c:7-95);
- the transpose (utils.h:158-195);
- A's tile structure (main_spgemm-col.cu:44-120);
- C's tile structure and tile contents (step1-step4, main_spgemm-col.cu:
  122-188, :572-627, :899-994, :4073-4179).

Structure must be identical.  Values must be identical for integer-valued
inputs, and otherwise within 1e-12 * sum|a||b| per entry.

Without the built reference (e.g. on a GPU host) the module is skipped;
the committed fixtures (test_oracle_golden.py) pin the oracle there.
"""
import ctypes as C
import importlib.util

import numpy as np
import pytest

from conftest import GOLDEN, ROOT, assert_values_close
from oracle import oracle as O

REF = ROOT / "oracle" / "_ref"


def _load():
    try:
        th = C.CDLL(str(REF / "libthmkl_ref.so"))
        st = C.CDLL(str(REF / "libstir_ref.so"))
    except OSError as e:
        pytest.skip(f"the reference's CPU code is not built here ({e})")
    spec = importlib.util.spec_from_file_location("make_golden", GOLDEN / "make_golden.py")
    mg = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mg)
    return th, st, mg


@pytest.fixture(scope="module")
def ref():
    return _load()


def _cases():
    from tilespgemm_gb300 import matrices as M
    rng = np.random.default_rng(2024)
    out = []
    for i in range(10):
        m, n = int(rng.integers(1, 260)), int(rng.integers(1, 260))
        k = int(rng.integers(1, 12))
        A = M.random_sparse(m, n, k, seed=100 + i, empty_rows=0.15 if i % 3 == 0 else 0.0,
                            band=(max(1, n // 10) if i % 4 == 1 else None))
        out.append((f"rand{i}_{m}x{n}", A, "AAT"))
        if m == n:
            out.append((f"rand{i}_{m}_AA", A, "AA"))
    out.append(("lap23_AA", M.laplacian_2d(23), "AA"))
    out.append(("st27_4_AA", M.stencil_27(4, seed=3), "AA"))
    out.append(("rmat9_AAT", M.rmat(9, 6, seed=11), "AAT"))
    out.append(("one_entry_AAT", M.random_sparse(1, 1, 1, seed=5), "AAT"))
    out.append(("rows_empty_AAT", M.random_sparse(40, 70, 3, seed=6, empty_rows=0.9), "AAT"))
    return out


CASES = _cases()


def _integer_values(A):
    from tilespgemm_gb300.api import CSR
    return CSR(A.m, A.n, A.rowptr, A.col, (np.arange(A.nnz) % 10).astype(np.float64))


@pytest.mark.parametrize("exact", [False, True])
@pytest.mark.parametrize("case", CASES, ids=[c[0] for c in CASES])
def test_oracle_matches_reference_live(ref, case, exact):
    th, st, mg = ref
    from tilespgemm_gb300.api import CSR
    _, A, op = case
    A = CSR(A.m, A.n, np.asarray(A.rowptr, np.int64), np.asarray(A.col, np.int32), np.asarray(A.val, np.float64))
    if exact:
        A = _integer_values(A)
    if op == "AA":
        B = A
    else:
        B = mg.ref_transpose(st, A)
        tp, tr, tv = O.transpose(A)
        assert np.array_equal(tp, B.rowptr) and np.array_equal(tr, B.col) and np.array_equal(tv, B.val)
    ic, jc, c = mg.ref_thmkl(th, A, B)
    rp, col, val, bnd = O.spgemm(A, B, with_bound=True)
    assert np.array_equal(rp, ic.astype(np.int64)) and np.array_equal(col, jc)
    if exact:
        assert np.array_equal(val, c)
    else:
        assert_values_close(val, c, bnd)
    brp, bci = mg.ref_tile_structure(st, A)
    t = O.tile_csr(A)
    assert np.array_equal(t["blkrowptr"], brp) and np.array_equal(t["blkcolidx"], bci)
    steps = mg.ref_steps(st, A, B)
    ts = O.tile_spgemm(A, B)
    for k in ("blkrowptrC", "blkcolidxC", "nnzbC", "ptrC", "colC"):
        assert np.array_equal(ts[{"blkrowptrC": "blkrowptr", "blkcolidxC": "blkcolidx", "nnzbC": "nnzb",
                                  "ptrC": "ptr", "colC": "col"}[k]], steps[k]), k
    if exact:
        assert np.array_equal(ts["val"], steps["valC"])
    else:
        assert np.allclose(ts["val"], steps["valC"], rtol=1e-12, atol=1e-13)
