"""Parity at the full sizes of the two large benchmark workloads.

* 3D 27-point stencil 96^3, C = A*A (884,736 rows, 622.8 M products,
  106.5 M entries of C): the whole C -- row pointer, columns, values -- is
  compared bit for bit with the oracle (same accumulation order, same FMA
  rounding as the CUDA path).
* R-MAT 2^20 x 16/row, C = A*A^T (about 2.1e10 products and 9.7e9 entries
  of C, 116 GB: too large to bring back or to compute whole on the CPU).
  C stays on the device; its whole row pointer comes back (int64: C has
  more than 2^31 entries), and about 2,000 rows -- the 20 with the most
  products (hub rows), 200 empty rows of A and a seeded random set -- come
  back through tsg_csr_download_rows and are compared with the oracle's
  row-subset product (structure bit for bit, values within
  1e-12 * sum|a||b| per entry and bit for bit as the design states).
"""
import numpy as np
import pytest

from conftest import assert_values_close
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def test_st27_96_whole_c_bit_exact():
    from tilespgemm_gb300 import Context
    from tilespgemm_gb300 import matrices as M
    A = M.stencil_27(96, seed=1)
    with Context(0) as ctx:
        C, st = ctx.spgemm(A, op="AA", stats=True)
    assert st["nnz_c"] == 106_496_424 and st["nnz_cub"] == 622_835_864
    rp, col, val = O.spgemm(A, A)
    assert np.array_equal(np.asarray(C.rowptr, np.int64), rp)
    assert np.array_equal(C.col, col)
    assert np.array_equal(C.val.view(np.int64), val.view(np.int64))


def _sample_rows(A, B, seed=7):
    rp = np.asarray(A.rowptr, np.int64)
    blen = np.diff(np.asarray(B.rowptr, np.int64))
    alen = np.diff(rp)
    per_entry = blen[np.asarray(A.col)].astype(np.int64)
    prod = np.zeros(A.m, np.int64)
    nz = alen > 0
    prod[nz] = np.add.reduceat(per_entry, rp[:-1][nz])
    rng = np.random.default_rng(seed)
    hubs = np.argsort(-prod, kind="stable")[:20]
    empty = np.flatnonzero(alen == 0)
    rows = np.concatenate([hubs, empty[rng.choice(empty.size, min(200, empty.size), replace=False)],
                           rng.choice(A.m, 1780, replace=False)])
    return np.unique(rows), hubs, prod


@pytest.fixture(scope="module")
def rmat20():
    from tilespgemm_gb300 import matrices as M
    from tilespgemm_gb300.api import CSR
    A = M.rmat(20, 16, seed=1)
    tp, tr, tv = O.transpose(A)
    return A, CSR(A.n, A.m, tp, tr, tv)


def test_rmat20_aat_sampled_rows(rmat20):
    from tilespgemm_gb300 import Context
    A, B = rmat20
    rows, hubs, prod = _sample_rows(A, B)
    crp_o, ccol_o, cval_o, bnd_o = O.spgemm_rows(A, B, rows)
    with Context(0) as ctx:
        oc, st = ctx.spgemm_raw(A, op="AAT", out="device", stats=True)
        try:
            assert st["nnz_cub"] == int(prod.sum())
            assert oc.rowptr_bits == 64 and oc.nnz == st["nnz_c"] and oc.nnz >= 2 ** 31
            rp = oc.rowptr()
            assert rp[0] == 0 and rp[-1] == oc.nnz and np.all(np.diff(rp) >= 0)
            # rows with no products are empty in C; rows with products are not
            assert np.array_equal(np.diff(rp) == 0, prod == 0)
            for t, r in enumerate(rows):
                lo, hi = crp_o[t], crp_o[t + 1]
                assert rp[r + 1] - rp[r] == hi - lo, f"row {r}: {rp[r + 1] - rp[r]} entries, oracle {hi - lo}"
                if hi == lo:
                    continue
                _, col, val = oc.rows(int(r), int(r) + 1)
                assert np.array_equal(col, ccol_o[lo:hi]), f"row {r}: columns differ"
                assert_values_close(val, cval_o[lo:hi], bnd_o[lo:hi])
                assert np.array_equal(val.view(np.int64), cval_o[lo:hi].view(np.int64)), f"row {r}: values differ"
        finally:
            oc.free()
    assert crp_o[-1] > 10_000_000   # the hub rows are in the sample


def test_rmat20_aat_int32_row_pointers_refused(rmat20):
    """C has more than 2^31 entries: a caller who asks for int32 row
    pointers gets TSG_ERR_INT32_OVERFLOW (before any work on C), and the
    context goes on working."""
    from tilespgemm_gb300 import Context, TSGError
    from tilespgemm_gb300 import _abi
    A, _ = rmat20
    with Context(0, out_rowptr_bits=32) as ctx:
        with pytest.raises(TSGError) as e:
            ctx.spgemm_raw(A, op="AAT", out="device")
        assert e.value.status == _abi.ERR_INT32_OVERFLOW
        from tilespgemm_gb300 import matrices as M
        L = M.laplacian_2d(64)
        C = ctx.spgemm(L, op="AA")
        rp, col, val = O.spgemm(L, L)
        assert np.array_equal(np.asarray(C.rowptr, np.int64), rp) and np.array_equal(C.val, val)
