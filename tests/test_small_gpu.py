"""The small-product path of tsg_spgemm (tsg_opts.small_path, default on):
A*B and A*A whose every row of A meets at most 128 entries of B run row by
row, one warp per row of C.  Its C must equal the oracle's and the tiled
pipeline's bit for bit (row pointer, columns, values: both accumulate each
entry as fma over A's row order, then B's); a repeated shape waits on the
device once per call; rows over the limit and A*A^T take the tiled path."""
import numpy as np
import pytest

from conftest import golden_names, load_case
from oracle import oracle as O

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def sctx(built_lib):
    from tilespgemm_gb300 import Context
    c = Context(0, small_path=1)
    yield c
    c.close()


def _same(C, D):
    assert C.m == D.m and C.n == D.n
    assert np.array_equal(np.asarray(C.rowptr, np.int64), np.asarray(D.rowptr, np.int64))
    assert np.array_equal(C.col, D.col)
    assert np.array_equal(C.val, D.val)


def _oracle(C, A, B):
    rp, col, val = O.spgemm(A, B)
    assert np.array_equal(np.asarray(C.rowptr, np.int64), rp)
    assert np.array_equal(C.col, col)
    assert np.array_equal(C.val, val)


def _banded_and_spread(m, k, seed):
    """Two m x m matrices with k entries in every row (the same shape): a
    band (C rows of about 2k entries) and random columns (about k^2)."""
    from tilespgemm_gb300.api import CSR
    rng = np.random.default_rng(seed)
    rp = np.arange(0, m * k + 1, k, dtype=np.int64)
    band = (np.arange(m)[:, None] + np.arange(k)[None, :]) % m
    band.sort(axis=1)
    spread = np.stack([np.sort(rng.choice(m, size=k, replace=False)) for _ in range(m)])
    vals = rng.uniform(-1.0, 1.0, size=m * k)
    return (CSR(m, m, rp, band.reshape(-1).astype(np.int32), vals),
            CSR(m, m, rp.copy(), spread.reshape(-1).astype(np.int32), vals.copy()))


def _cases():
    from tilespgemm_gb300 import matrices as M
    return {
        "lap64": (M.laplacian_2d(64), None, "AA"),
        "lap256": (M.laplacian_2d(256), None, "AA"),
        "rand5000": (M.random_sparse(5000, 5000, 10, seed=12), None, "AA"),
        "dups_unsorted": (M.random_sparse(1000, 1000, 8, seed=15, dup=True, unsorted=True), None, "AA"),
        "empty_rows": (M.random_sparse(3000, 3000, 6, seed=16, empty_rows=0.5), None, "AA"),
        "rect_ab": (M.random_sparse(300, 500, 9, seed=21), M.random_sparse(500, 170, 7, seed=22), "AB"),
        "far_columns": (M.random_sparse(200, 100000, 8, seed=5), M.random_sparse(100000, 90000, 8, seed=6), "AB"),
        "full_rows": (M.random_sparse(64, 64, 11, seed=7), None, "AA"),
    }


@pytest.mark.parametrize("key", list(_cases().keys()))
def test_small_path_matches_oracle_and_tiled(sctx, ctx, key):
    A, B, op = _cases()[key]
    C, st = sctx.spgemm(A, B, op=op, stats=True)
    assert st["small_path"] == 1
    _oracle(C, A, B if B is not None else A)
    T, st2 = ctx.spgemm(A, B, op=op, stats=True)
    assert st2["small_path"] == 0
    _same(C, T)
    assert st["nnz_c"] == C.nnz and st["nnz_cub"] == O.nnzcub(A, B if B is not None else A)


@pytest.mark.parametrize("name", [n for n in golden_names() if load_case(n)["op"] != "AAT"])
def test_small_path_golden(sctx, name):
    d = load_case(name)
    C, st = sctx.spgemm(d["A"], op=d["op"], stats=True)
    assert np.array_equal(np.asarray(C.rowptr, np.int64), d["c_rowptr"])
    assert np.array_equal(C.col, d["c_col"])
    _oracle(C, d["A"], d["B"])


def test_repeated_shape_waits_once(built_lib):
    """A shape's first call counts, scans, reads C's size back and fills (two
    waits); a repeat with the same structure fills at the kept row pointer
    and waits once; a matrix of the same shape but another structure is
    caught there (every row is counted again), counted and filled into
    buffers sized from the last call -- and filled once more when C
    outgrew them -- with the exact result every time."""
    from tilespgemm_gb300 import Context
    band, spread = _banded_and_spread(3000, 8, seed=3)

    def run(c, X, Xd, syncs):
        oc, st = c.spgemm_raw(Xd, op="AA", out="device", stats=True)
        C = oc.download()
        oc.free()
        _oracle(C, X, X)
        assert st["small_path"] == 1 and st["n_syncs"] == syncs, st["n_syncs"]
        assert st["nnz_cub"] == O.nnzcub(X, X)

    with Context(0) as c:
        Ad, Sd = band.to_device(0), spread.to_device(0)
        run(c, band, Ad, 2)
        run(c, band, Ad, 1)
        run(c, band, Ad, 1)
        run(c, spread, Sd, 3)      # kept fill, count + fill, fill again (C about 4x larger)
        run(c, spread, Sd, 1)
        run(c, band, Ad, 2)        # kept fill, count + fill (the buffers are large enough)
        run(c, band, Ad, 1)


def test_one_round_shape_then_longer_rows(built_lib):
    """A shape whose rows all fit one warp round (at most 32 products) runs
    the register-only fill when repeated; the same shape with rows of more
    products is caught there, counted again and filled by the general
    kernel -- exact every time."""
    from tilespgemm_gb300 import Context
    from tilespgemm_gb300.api import CSR
    rng = np.random.default_rng(61)

    def rows(lens, n):
        rp = np.zeros(len(lens) + 1, np.int64)
        np.cumsum(lens, out=rp[1:])
        col = np.concatenate([np.sort(rng.choice(n, size=int(L), replace=False)) for L in lens]).astype(np.int32)
        return CSR(len(lens), n, rp, col, rng.uniform(-1.0, 1.0, size=col.size))

    A = rows([5] * 2000, 1000)
    B1 = rows([5] * 1000, 800)                               # 25 products per row of A
    B2 = rows([20] * 10 + [5] * 840 + [4] * 150, 800)         # the same nnz; rows 0-9 of 20 entries
    assert B1.nnz == B2.nnz
    with Context(0) as c:
        Ad, B1d, B2d = A.to_device(0), B1.to_device(0), B2.to_device(0)
        for B, Bd, syncs in ((B1, B1d, 2), (B1, B1d, 1), (B2, B2d, None), (B2, B2d, 1), (B1, B1d, None)):
            oc, st = c.spgemm_raw(Ad, Bd, op="AB", out="device", stats=True)
            C = oc.download()
            oc.free()
            _oracle(C, A, B)
            assert st["small_path"] == 1
            if syncs is not None:
                assert st["n_syncs"] == syncs
            else:
                assert st["n_syncs"] >= 2


def test_wide_b_uses_long_sort_keys(sctx, ctx):
    """B with more than 2^26 columns: the one-round sort keys (column, product
    index) take 64 bits.  Columns drawn from a small shared pool spread over
    80 M so that products meet; the result equals the tiled path's bit for
    bit (both accumulate in A's order, then B's)."""
    from tilespgemm_gb300.api import CSR
    rng = np.random.default_rng(71)
    pool = np.sort(rng.choice(80_000_000, size=300, replace=False))

    def rows(m, n, per, choose):
        rp = np.arange(0, m * per + 1, per, dtype=np.int64)
        col = np.concatenate([np.sort(choose()) for _ in range(m)]).astype(np.int32)
        return CSR(m, n, rp, col, rng.uniform(-1.0, 1.0, size=col.size))

    A = rows(400, 1000, 4, lambda: rng.choice(1000, size=4, replace=False))
    B = rows(1000, 80_000_000, 8, lambda: rng.choice(pool, size=8, replace=False))
    C, st = sctx.spgemm(A, B, op="AB", stats=True)
    assert st["small_path"] == 1
    T = ctx.spgemm(A, B, op="AB")
    _same(C, T)
    assert C.nnz < 400 * 32   # products met


def test_rows_over_the_limit_take_the_tiled_path(sctx):
    from tilespgemm_gb300 import matrices as M
    A = M.random_sparse(500, 500, 12, seed=40)      # 144 products per row
    for _ in range(2):
        C, st = sctx.spgemm(A, op="AA", stats=True)
        assert st["small_path"] == 0
        _oracle(C, A, A)
    R = M.rmat(9, 8, seed=2)
    C, st = sctx.spgemm(R, op="AAT", stats=True)
    assert st["small_path"] == 0


@pytest.mark.parametrize("op", ["AA", "AB"])
def test_pinned_host_operands_and_output(sctx, op):
    import torch
    from tilespgemm_gb300 import matrices as M
    from tilespgemm_gb300.api import CSR

    def pinned(X):
        return CSR(X.m, X.n, torch.from_numpy(np.asarray(X.rowptr, np.int64)).pin_memory(),
                   torch.from_numpy(np.asarray(X.col, np.int32)).pin_memory(),
                   torch.from_numpy(np.asarray(X.val, np.float64)).pin_memory())

    A = M.random_sparse(4000, 3000, 7, seed=50, empty_rows=0.1)
    B = M.random_sparse(3000, 2500, 9, seed=51) if op == "AB" else None
    if op == "AA":
        A = M.random_sparse(4000, 4000, 7, seed=50, empty_rows=0.1)
    for _ in range(2):
        oc, st = sctx.spgemm_raw(pinned(A), pinned(B) if B is not None else None, op=op, out="host", stats=True)
        assert oc.where == "host" and st["small_path"] == 1
        C = oc.download()
        oc.free()
        _oracle(C, A, B if B is not None else A)


def test_int64_row_pointers_and_tiny(built_lib):
    from tilespgemm_gb300 import Context
    from tilespgemm_gb300 import matrices as M
    from tilespgemm_gb300.api import CSR
    A = M.laplacian_2d(40)
    with Context(0, out_rowptr_bits=64) as c:
        oc, st = c.spgemm_raw(A.to_device(0), op="AA", out="device", stats=True)
        assert oc.rowptr_bits == 64 and st["small_path"] == 1
        C = oc.download()
        oc.free()
        _oracle(C, A, A)
        Z = CSR(40, 40, np.zeros(41, np.int64), np.zeros(0, np.int32), np.zeros(0))
        C = c.spgemm(Z, op="AA")
        assert C.nnz == 0 and np.all(np.asarray(C.rowptr) == 0)
        one = CSR(1, 1, np.array([0, 1]), np.array([0], np.int32), np.array([3.0]))
        C = c.spgemm(one, op="AA")
        assert C.nnz == 1 and C.val[0] == 9.0
        E = CSR(0, 0, np.zeros(1, np.int64), np.zeros(0, np.int32), np.zeros(0))
        C = c.spgemm(E, op="AA")
        assert C.m == 0 and C.nnz == 0


def test_invalid_inputs_are_reported(sctx):
    """The same statuses as the tiled path, on a first call of a shape and on
    a repeated one; the context stays usable."""
    from tilespgemm_gb300 import TSGError
    from tilespgemm_gb300.api import CSR
    good = CSR(3, 3, np.array([0, 1, 2, 3]), np.array([0, 2, 1], np.int32), np.ones(3))
    bad_col = CSR(3, 3, np.array([0, 1, 2, 3]), np.array([0, 5, 1], np.int32), np.ones(3))
    bad_rp = CSR(3, 3, np.array([0, 2, 1, 3]), np.array([0, 1, 2], np.int32), np.ones(3))
    for first in (True, False):
        if not first:
            sctx.spgemm(good, op="AA")      # the shape is known now
        for bad in (bad_col, bad_rp):
            with pytest.raises(TSGError) as e:
                sctx.spgemm(bad, op="AA")
            assert e.value.status == 8
    rect = CSR(2, 3, np.array([0, 1, 2]), np.array([0, 2], np.int32), np.ones(2))
    with pytest.raises(TSGError) as e:
        sctx.spgemm(rect, op="AA")
    assert e.value.status == 7
    ok = CSR(2, 2, np.array([0, 1, 2]), np.array([1, 0], np.int32), np.array([2.0, 3.0]))
    C = sctx.spgemm(ok, op="AA")
    assert np.array_equal(C.val, [6.0, 6.0])


def test_invalid_ab_operands_on_a_repeated_shape(sctx):
    """A repeated A*B shape runs the fill alone on the operands as given and
    validates them there: a column of B out of range in a row that A never
    reaches, a B row pointer out of order, a column of A out of range --
    each TSG_ERR_BAD_INPUT, as from the validation kernel -- and the
    context stays exact."""
    from tilespgemm_gb300 import TSGError
    from tilespgemm_gb300.api import CSR
    A = CSR(3, 3, np.array([0, 1, 2, 3]), np.array([0, 0, 1], np.int32), np.array([1.0, 2.0, 3.0]))
    B = CSR(3, 4, np.array([0, 2, 3, 4]), np.array([0, 3, 1, 2], np.int32), np.array([1.0, 2.0, 3.0, 4.0]))
    ref = O.spgemm(A, B)
    for _ in range(2):
        C = sctx.spgemm(A, B, op="AB")
        assert np.array_equal(C.col, ref[1]) and np.array_equal(C.val, ref[2])
    bad_b_col = CSR(3, 4, B.rowptr, np.array([0, 3, 1, 7], np.int32), B.val)      # row 2: A never reads it
    bad_b_rp = CSR(3, 4, np.array([0, 3, 2, 4]), B.col, B.val)
    bad_a_col = CSR(3, 3, A.rowptr, np.array([0, 5, 1], np.int32), A.val)
    for a, b in ((A, bad_b_col), (A, bad_b_rp), (bad_a_col, B)):
        with pytest.raises(TSGError) as e:
            sctx.spgemm(a, b, op="AB")
        assert e.value.status == 8
    C = sctx.spgemm(A, B, op="AB")
    assert np.array_equal(C.col, ref[1]) and np.array_equal(C.val, ref[2])


def test_allocation_failures_are_reported(built_lib):
    """Every device-pool allocation of a small-path call, on a first call of
    the shape and on a repeated one, fails in turn: TSG_ERR_OOM, and the next
    call is exact."""
    from tilespgemm_gb300 import Context, _abi
    from tilespgemm_gb300 import matrices as M
    from test_failure_gpu import _sweep
    A = M.random_sparse(900, 900, 9, seed=31, empty_rows=0.1)

    def first_call():                      # a new context: the shape is not known yet
        with Context(0, small_path=1) as c2:
            C, st = c2.spgemm(A, op="AA", stats=True)
            assert st["small_path"] == 1
            _oracle(C, A, A)

    c = Context(0, small_path=1)
    try:
        def call():
            C, st = c.spgemm(A, op="AA", stats=True)
            assert st["small_path"] == 1
            _oracle(C, A, A)

        assert _sweep(0, first_call, first_call) >= 5
        assert _sweep(0, call, call) >= 5  # the shape is known after the first successful call
        assert _sweep(1, lambda: c.spgemm(A, op="AA"), call) >= 3   # pinned host buffers of C
    finally:
        _abi.lib().tsg_inject_alloc_failure(0, 0)
        _abi.lib().tsg_inject_alloc_failure(1, 0)
        c.close()
