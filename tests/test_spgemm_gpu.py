"""GPU parity: the CUDA path (through the C ABI) against the oracle and the
reference goldens.  Structure is compared bit for bit; values bit for bit
against the oracle (same accumulation order, same FMA rounding) and within
1e-12 * sum|a||b| per entry against the reference CPU path."""
import numpy as np
import pytest

from conftest import assert_values_close, golden_names, load_case
from oracle import oracle as O

pytestmark = pytest.mark.gpu
CASES = golden_names()


def check_against_oracle(C, A, B, exact=True):
    rp, col, val, bnd = O.spgemm(A, B, with_bound=True)
    assert C.m == A.m and C.n == B.n
    assert np.array_equal(np.asarray(C.rowptr, np.int64), rp)
    assert np.array_equal(C.col, col)
    if exact:
        assert np.array_equal(C.val, val), np.max(np.abs(C.val - val)) if val.size else 0
    else:
        assert_values_close(C.val, val, bnd)


@pytest.mark.parametrize("name", CASES)
def test_csr_matches_golden(ctx, name):
    d = load_case(name)
    C = ctx.spgemm(d["A"], op=d["op"])
    assert np.array_equal(np.asarray(C.rowptr, np.int64), d["c_rowptr"])
    assert np.array_equal(C.col, d["c_col"])
    if d["exact"]:
        assert np.array_equal(C.val, d["c_val"])
    else:
        _, _, _, bnd = O.spgemm(d["A"], d["B"], with_bound=True)
        assert_values_close(C.val, d["c_val"], bnd)
    check_against_oracle(C, d["A"], d["B"])


@pytest.mark.parametrize("name", CASES)
def test_tiles_match_reference_steps(ctx, name):
    """C's tile form equals the reference's step1..step4 output, including the
    structurally empty tiles (nnz 0, mask 0, row starts 0)."""
    d = load_case(name)
    T = ctx.spgemm_tiles(d["A"], op=d["op"])
    assert np.array_equal(T.blkrowptr, d["blkrowptrC"].astype(np.int64))
    assert np.array_equal(T.blkcolidx, d["blkcolidxC"])
    assert np.array_equal(T.nnzb, d["nnzbC"].astype(np.int64))
    assert np.array_equal(T.ptr, d["ptrC"])
    assert np.array_equal(T.col, d["colC"])
    if d["exact"]:
        assert np.array_equal(T.val, d["valC"])
    else:
        assert np.allclose(T.val, d["valC"], rtol=1e-12, atol=1e-13)
    ref_mask = O.tile_spgemm(d["A"], d["B"])["mask"]
    assert np.array_equal(T.mask, ref_mask)


@pytest.mark.parametrize("name", CASES)
def test_csr_to_tiles_matches_oracle(ctx, name):
    d = load_case(name)
    T = ctx.csr_to_tiles(d["A"])
    t = O.tile_csr(d["A"])
    assert np.array_equal(T.blkrowptr, t["blkrowptr"].astype(np.int64))
    assert np.array_equal(T.blkcolidx, t["blkcolidx"])
    assert np.array_equal(T.nnzb, t["nnzb"].astype(np.int64))
    assert np.array_equal(T.ptr, t["ptr"])
    assert np.array_equal(T.col, t["lcol"])
    assert np.array_equal(T.val, t["val"])
    assert np.array_equal(T.mask, t["mask"])
    assert np.array_equal(T.blkcolidx, d["a_blkcolidx"])


@pytest.mark.parametrize("name", [n for n in CASES if "unsorted" not in n])
def test_tiles_roundtrip(ctx, name):
    d = load_case(name)
    A = d["A"]
    R = ctx.tiles_roundtrip(A)
    assert np.array_equal(R.rowptr, A.rowptr)
    assert np.array_equal(R.col, A.col)
    assert np.array_equal(R.val, A.val)


def _mats():
    from tilespgemm_gb300 import matrices as M
    return {
        "lap64": (M.laplacian_2d(64), "AA"),
        "lap256": (M.laplacian_2d(256), "AA"),
        "st27_20": (M.stencil_27(20, seed=3), "AA"),
        "rand5000": (M.random_sparse(5000, 5000, 10, seed=12), "AA"),
        "band4000": (M.random_sparse(4000, 4000, 24, seed=13, band=100), "AA"),
        "rmat12_aat": (M.rmat(12, 16, seed=5), "AAT"),
        "rmat12_aa": (M.rmat(12, 8, seed=6), "AA"),
        "rect_aat": (M.random_sparse(700, 2500, 12, seed=14), "AAT"),
        "dups": (M.random_sparse(1000, 1000, 20, seed=15, dup=True, unsorted=True), "AA"),
        "empty_rows": (M.random_sparse(3000, 3000, 6, seed=16, empty_rows=0.5), "AA"),
        "long_rows": (M.random_sparse(64, 64, 60, seed=17), "AA"),
    }


@pytest.mark.parametrize("key", list(_mats().keys()))
def test_random_matrices_bit_exact(ctx, key):
    A, op = _mats()[key]
    B = A if op == "AA" else O_transpose_csr(A)
    C = ctx.spgemm(A, op=op)
    check_against_oracle(C, A, B)


def O_transpose_csr(A):
    from tilespgemm_gb300.api import CSR
    tp, tr, tv = O.transpose(A)
    return CSR(A.n, A.m, tp, tr, tv)


def _mixed_b(k, n, seed):
    """B with mostly 3-entry rows and every 37th row 200 entries long."""
    from tilespgemm_gb300 import matrices as M
    rng = np.random.default_rng(seed)
    lens = np.where(np.arange(k) % 37 == 0, min(200, n), 3)
    r = np.repeat(np.arange(k, dtype=np.int64), lens)
    c = np.concatenate([rng.choice(n, size=int(L), replace=False) for L in lens])
    return M._from_coo(k, n, r, c, rng.uniform(-1.0, 1.0, size=r.size), merge=True)


@pytest.mark.parametrize("n", [900, 9000])
def test_sparse_a_tiles_mixed_b_rows(ctx, n):
    """A tiles of about one entry (the symbolic steps walk A by entry) times
    B rows both shorter and longer than the entry walk takes (the long ones
    go through B's tile masks); C tile-rows narrow (n=900) and wide (n=9000)."""
    from tilespgemm_gb300 import matrices as M
    A = M.random_sparse(2000, 3000, 4, seed=31)
    B = _mixed_b(3000, n, seed=32)
    C = ctx.spgemm(A, B, op="AB")
    check_against_oracle(C, A, B)


def test_general_ab_rectangular(ctx):
    from tilespgemm_gb300 import matrices as M
    A = M.random_sparse(300, 500, 9, seed=21)
    B = M.random_sparse(500, 170, 7, seed=22)
    C = ctx.spgemm(A, B, op="AB")
    check_against_oracle(C, A, B)


@pytest.mark.parametrize("opts", [dict(smem_acc_max=0), dict(smem_acc_max=0, row_acc_max=0), dict(dense_tile_min=1),
                                  dict(threads_numeric=128), dict(threads_numeric=512), dict(out_rowptr_bits=64),
                                  dict(numeric_walk=1), dict(numeric_walk=2), dict(numeric_walk=3), dict(numeric_walk=2, dense_tile_min=1),
                                  dict(numeric_walk=3, dense_tile_min=1),
                                  dict(smem_acc_max=0, row_warps=1), dict(smem_acc_max=0, numeric_walk=2)])
def test_numeric_bins_agree(opts, built_lib):
    """Every accumulator path (shared sparse, shared dense, one row per CTA,
    global) gives the same bits."""
    from tilespgemm_gb300 import Context
    from tilespgemm_gb300 import matrices as M
    A = M.stencil_27(12, seed=4)
    B2 = M.random_sparse(2000, 2000, 15, seed=23, dup=True)
    B3 = M.random_sparse(3000, 3000, 12, seed=25, band=24)   # few C tiles per tile-row
    with Context(0, small_path=0, **opts) as c:
        for X in (A, B2, B3):
            C, st = c.spgemm(X, op="AA", stats=True)
            check_against_oracle(C, X, X)
            if opts.get("smem_acc_max") == 0:
                assert st["bins"][3] > 0
            if opts.get("dense_tile_min") == 1 and X is B3:
                assert st["bins"][2] > 0
            if opts.get("out_rowptr_bits") == 64:
                assert C.rowptr.dtype == np.int64


@pytest.mark.parametrize("opts", [dict(), dict(row_warps=1), dict(row_warps=2), dict(row_acc_max=0), dict(rows_global=1)])
def test_long_rows(opts, built_lib):
    """C rows of ~3,900 and ~8,400 entries: the medium and large size classes
    of the one-row-per-CTA kernel (and, with row_acc_max=0, the global
    accumulator), bit-exact against the oracle."""
    from tilespgemm_gb300 import Context
    from tilespgemm_gb300 import matrices as M
    with Context(0, small_path=0, **opts) as c:
        for X in (M.random_sparse(6000, 6000, 80, seed=31), M.random_sparse(12000, 12000, 120, seed=32)):
            C, st = c.spgemm(X, op="AA", stats=True)
            assert st["bins"][3] > 0
            check_against_oracle(C, X, X)


@pytest.mark.parametrize("opts", [dict(smem_acc_max=0, row_acc_max=0), dict()])
def test_hub_rows_in_parts(opts, built_lib):
    """A rows of ~590 entries times B spread over 300,000 columns: with every
    row sent to the wide class (smem_acc_max=0, row_acc_max=0) the rows of
    long A rows are cut into parts walked anywhere on the GPU from a table
    of B-row cut points; bit-exact against the oracle either way."""
    from tilespgemm_gb300 import Context
    from tilespgemm_gb300 import matrices as M
    A = M.random_sparse(48, 2000, 700, seed=41)
    B = M.random_sparse(2000, 300000, 20, seed=42)
    assert int(np.diff(np.asarray(A.rowptr)).min()) > 512
    with Context(0, small_path=0, **opts) as c:
        C, st = c.spgemm(A, B, op="AB", stats=True)
        assert st["bins"][3] > 0
        check_against_oracle(C, A, B)


def _runs_matrix(m, n, runs, seed):
    """Row k holds the column runs given by runs(k) -> list of (start, length),
    values uniform in [-1, 1]."""
    from tilespgemm_gb300.api import CSR
    rng = np.random.default_rng(seed)
    rp, cols = [0], []
    for k in range(m):
        c = np.unique(np.concatenate([np.arange(s0, min(s0 + ln, n)) for s0, ln in runs(k)]))
        cols.append(c)
        rp.append(rp[-1] + c.size)
    col = np.concatenate(cols).astype(np.int32)
    return CSR(m, n, np.array(rp, np.int64), col, rng.uniform(-1, 1, col.size))


@pytest.mark.parametrize("opts", [dict(), dict(dense_tile_min=257)])
def test_wide_tile_rows(ctx, opts, built_lib):
    """C tile-rows with more than 2,048 tiles (windowed step 2) and rows
    spanning more than 4,096 tile columns (windowed global accumulator):
    dense tiles (tile path) and scattered entries (element path)."""
    from tilespgemm_gb300 import Context
    A = _runs_matrix(32, 120, lambda k: [(0, 120)], seed=41)                       # dense rows
    B1 = _runs_matrix(120, 120000, lambda k: [(k * 1000, 300)], seed=42)            # dense tiles
    B2 = _runs_matrix(120, 120000, lambda k: [(k * 997 + 16 * t, 1) for t in range(300)], seed=43)  # 1 per tile
    with Context(0, small_path=0, **opts) as c:
        for B in (B1, B2):
            C, st = c.spgemm(A, B, op="AB", stats=True)
            assert st["bins"][3] > 0
            check_against_oracle(C, A, B)


def test_device_inputs_and_outputs(ctx):
    import torch
    from tilespgemm_gb300 import matrices as M
    A = M.random_sparse(2000, 2000, 8, seed=24)
    Ad = A.to_device(0)
    oc, st = ctx.spgemm_raw(Ad, op="AA", out="device", stats=True)
    assert oc.where == "device"
    C = oc.download()
    oc.free()
    check_against_oracle(C, A, A)
    assert st["nnz_cub"] == O.nnzcub(A, A)
    A32 = A.to_device(0)
    A32.rowptr = A32.rowptr.to(torch.int32)
    C2 = ctx.spgemm(A32, op="AA")
    assert np.array_equal(C2.col, C.col) and np.array_equal(C2.val, C.val)


@pytest.mark.parametrize("op", ["AA", "AB", "AAT"])
def test_pinned_host_operands_and_output(ctx, op):
    """Host operands in pinned memory (values go up on the copy stream while
    the symbolic phase runs) and host output (C's column indices come down
    while the numeric step runs; C tiles of 8 entries or more on average):
    narrow tile-rows and tile-rows of more than 32 C tiles, bit-exact
    against the oracle and the device path."""
    import torch
    from tilespgemm_gb300 import matrices as M
    from tilespgemm_gb300.api import CSR

    def pinned(X):
        return CSR(X.m, X.n, torch.from_numpy(np.asarray(X.rowptr, np.int64)).pin_memory(),
                   torch.from_numpy(np.asarray(X.col, np.int32)).pin_memory(),
                   torch.from_numpy(np.asarray(X.val, np.float64)).pin_memory())

    mats = [M.laplacian_2d(64), M.stencil_27(12, seed=3), M.random_sparse(700, 700, 60, seed=8, empty_rows=0.05)]
    for A in mats:
        B = M.random_sparse(A.n, 900, 12, seed=9) if op == "AB" else None
        Bt = B if op == "AB" else (A if op == "AA" else O_transpose_csr(A))
        oc, _ = ctx.spgemm_raw(pinned(A), pinned(B) if B is not None else None, op=op, out="host")
        assert oc.where == "host"
        C = oc.download()
        oc.free()
        check_against_oracle(C, A, Bt)
        Cd = ctx.spgemm_raw(A.to_device(0), B.to_device(0) if B is not None else None, op=op, out="device")[0]
        C2 = Cd.download()
        Cd.free()
        assert np.array_equal(np.asarray(C2.rowptr, np.int64), np.asarray(C.rowptr, np.int64))
        assert np.array_equal(C2.col, C.col) and np.array_equal(C2.val, C.val)


def test_stats_and_syncs(ctx):
    from tilespgemm_gb300 import matrices as M
    A = M.laplacian_2d(100)
    C, st = ctx.spgemm(A, op="AA", stats=True)
    assert st["nnz_c"] == C.nnz and st["nnz_a"] == A.nnz
    assert st["nnz_cub"] == O.nnzcub(A, A)
    assert st["n_syncs"] <= 3
    assert st["tiles_a"] == O.tile_csr(A)["numblk"]


def test_empty_and_tiny(ctx):
    from tilespgemm_gb300.api import CSR
    Z = CSR(40, 40, np.zeros(41, np.int64), np.zeros(0, np.int32), np.zeros(0))
    C = ctx.spgemm(Z, op="AA")
    assert C.nnz == 0 and np.all(C.rowptr == 0)
    one = CSR(1, 1, np.array([0, 1]), np.array([0], np.int32), np.array([3.0]))
    C = ctx.spgemm(one, op="AA")
    assert C.nnz == 1 and C.val[0] == 9.0
    E = CSR(0, 0, np.zeros(1, np.int64), np.zeros(0, np.int32), np.zeros(0))
    C = ctx.spgemm(E, op="AA")
    assert C.m == 0 and C.nnz == 0


def test_cancellation_keeps_structural_zero(ctx):
    """An entry whose products cancel to 0.0 stays in C (the reference's flag
    is structural, thmkl_dcsrmultcsr.c:63-72)."""
    from tilespgemm_gb300.api import CSR
    A = CSR(2, 2, np.array([0, 2, 3]), np.array([0, 1, 0], np.int32), np.array([1.0, 1.0, 1.0]))
    B = CSR(2, 2, np.array([0, 1, 2]), np.array([0, 0], np.int32), np.array([1.0, -1.0]))
    C = ctx.spgemm(A, B, op="AB")
    assert np.array_equal(C.rowptr, [0, 1, 2]) and np.array_equal(C.col, [0, 0])
    assert C.val[0] == 0.0 and C.val[1] == 1.0


def test_invalid_inputs_are_reported(ctx):
    from tilespgemm_gb300 import TSGError
    from tilespgemm_gb300.api import CSR
    bad_col = CSR(3, 3, np.array([0, 1, 2, 3]), np.array([0, 5, 1], np.int32), np.ones(3))
    with pytest.raises(TSGError) as e:
        ctx.spgemm(bad_col, op="AA")
    assert e.value.status == 8
    bad_rp = CSR(3, 3, np.array([0, 2, 1, 3]), np.array([0, 1, 2], np.int32), np.ones(3))
    with pytest.raises(TSGError) as e:
        ctx.spgemm(bad_rp, op="AA")
    assert e.value.status == 8
    rect = CSR(2, 3, np.array([0, 1, 2]), np.array([0, 2], np.int32), np.ones(2))
    with pytest.raises(TSGError) as e:
        ctx.spgemm(rect, op="AA")
    assert e.value.status == 7
    # the context stays usable after errors
    ok = CSR(2, 2, np.array([0, 1, 2]), np.array([1, 0], np.int32), np.array([2.0, 3.0]))
    C = ctx.spgemm(ok, op="AA")
    assert np.array_equal(C.val, [6.0, 6.0])


def test_repeat_calls_reuse_pool(ctx):
    from tilespgemm_gb300 import matrices as M
    A = M.stencil_27(16, seed=9)
    first = ctx.spgemm(A, op="AA")
    for _ in range(3):
        again = ctx.spgemm(A, op="AA")
        assert np.array_equal(again.val, first.val) and np.array_equal(again.col, first.col)


def test_tiles_spmv(ctx):
    """y = T x on the tile form (tsg_tiles_spmv) of A and of C = A*A, against
    a CSR SpMV on the host (within 1e-12 of sum |t_ij x_j|)."""
    import ctypes as C
    import torch
    from tilespgemm_gb300 import _abi
    from tilespgemm_gb300 import matrices as M
    lib = _abi.lib()
    A = M.random_sparse(3000, 3000, 12, seed=51, empty_rows=0.05)
    rng = np.random.default_rng(7)
    x = rng.uniform(-1.0, 1.0, A.n)
    xd = torch.tensor(x, dtype=torch.float64, device="cuda")
    a, keep = A._tsg()
    Cref = O.spgemm(A, A)
    for which in ("A", "C"):
        t = _abi.tsg_tiles()
        if which == "A":
            _abi.check(lib.tsg_csr_to_tiles(ctx.handle, C.byref(a), C.byref(t)))
            rp, col, val = np.asarray(A.rowptr, np.int64), np.asarray(A.col), np.asarray(A.val)
        else:
            _abi.check(lib.tsg_spgemm_tiles(ctx.handle, _abi.OP_AA, C.byref(a), None, C.byref(t), None))
            rp, col, val = Cref[0], Cref[1], Cref[2]
        try:
            yd = torch.full((t.m,), float("nan"), dtype=torch.float64, device="cuda")
            _abi.check(lib.tsg_tiles_spmv(ctx.handle, C.byref(t), xd.data_ptr(), yd.data_ptr()))
            y = yd.cpu().numpy()
        finally:
            lib.tsg_tiles_free(ctx.handle, C.byref(t))
        rows = np.repeat(np.arange(len(rp) - 1), np.diff(rp))
        yref = np.bincount(rows, weights=val * x[col], minlength=len(rp) - 1)
        bound = np.bincount(rows, weights=np.abs(val * x[col]), minlength=len(rp) - 1)
        assert np.all(np.abs(y - yref) <= 1e-12 * bound + 1e-300)
    del keep


@pytest.mark.parametrize("kind", ["unsorted", "dup"])
def test_long_rows_unsorted_and_repeated(kind, built_lib):
    """Long rows (global accumulator, eight warps over column ranges) with B
    rows that are unsorted (every entry tested against the range) or repeat
    columns (the packed walk)."""
    from tilespgemm_gb300 import Context
    from tilespgemm_gb300 import matrices as M
    X = M.random_sparse(5000, 5000, 60, seed=33, unsorted=(kind == "unsorted"), dup=(kind == "dup"))
    with Context(0, small_path=0, row_acc_max=0) as c:
        C = c.spgemm(X, op="AA")
        check_against_oracle(C, X, X)
