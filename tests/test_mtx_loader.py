"""Matrix Market load path (tsg_load_mtx, host code in libtilespgemm.so)
against the reference loader mmio_allinone's outputs (mtx_*.npz)."""
import numpy as np
import pytest

from conftest import GOLDEN

FILES = sorted(p.stem for p in (GOLDEN / "mtx").glob("*.mtx"))


@pytest.mark.parametrize("stem", FILES)
def test_load_matches_reference(built_lib, stem):
    from tilespgemm_gb300 import TSGError, load_mtx
    g = np.load(GOLDEN / f"mtx_{stem}.npz")
    path = GOLDEN / "mtx" / f"{stem}.mtx"
    if int(g["rc"]) != 0:
        with pytest.raises(TSGError) as ei:
            load_mtx(path)
        assert ei.value.status == 5  # TSG_ERR_BAD_MTX
        return
    A, sym = load_mtx(path)
    assert (A.m, A.n, A.nnz, int(sym)) == (int(g["m"]), int(g["n"]), int(g["nnz"]), int(g["sym"]))
    assert np.array_equal(A.rowptr, g["rowptr"])
    assert np.array_equal(A.col, g["col"])
    assert np.array_equal(A.val, g["val"])


def test_missing_file(built_lib, tmp_path):
    from tilespgemm_gb300 import TSGError, load_mtx
    with pytest.raises(TSGError) as ei:
        load_mtx(tmp_path / "nope.mtx")
    assert ei.value.status == 5


def test_truncated_and_out_of_range(built_lib, tmp_path):
    from tilespgemm_gb300 import TSGError, load_mtx
    p = tmp_path / "t.mtx"
    p.write_text("%%MatrixMarket matrix coordinate real general\n3 3 2\n1 1 1.0\n")
    with pytest.raises(TSGError):
        load_mtx(p)
    p.write_text("%%MatrixMarket matrix coordinate real general\n3 3 1\n4 1 1.0\n")
    with pytest.raises(TSGError):
        load_mtx(p)
    p.write_text("%%MatrixMarket matrix array real general\n2 2\n1\n2\n3\n4\n")
    with pytest.raises(TSGError):
        load_mtx(p)


def test_roundtrip_generated(built_lib, tmp_path):
    """A generated matrix written as .mtx loads back to the same CSR."""
    from tilespgemm_gb300 import load_mtx
    from tilespgemm_gb300 import matrices as M
    A = M.random_sparse(50, 40, 4, seed=11)
    rows = np.repeat(np.arange(A.m), np.diff(A.rowptr))
    with open(tmp_path / "g.mtx", "w") as f:
        f.write("%%MatrixMarket matrix coordinate real general\n")
        f.write(f"{A.m} {A.n} {A.nnz}\n")
        for r, c, v in zip(rows, A.col, A.val):
            f.write(f"{r + 1} {c + 1} {float(v)!r}\n")
    B, sym = load_mtx(tmp_path / "g.mtx")
    assert not sym
    assert np.array_equal(B.rowptr, A.rowptr) and np.array_equal(B.col, A.col) and np.array_equal(B.val, A.val)


def test_write_then_load_round_trip(built_lib, tmp_path):
    """tsg_write_mtx: the reference writer's format (banner, size line,
    1-based 'i j %20.16g' lines in CSR order); exact mode loads back bit for
    bit."""
    from tilespgemm_gb300 import load_mtx, write_mtx
    from tilespgemm_gb300 import matrices as M
    A = M.random_sparse(37, 23, 4, seed=3)
    p = tmp_path / "a.mtx"
    write_mtx(p, A)
    lines = p.read_text().splitlines()
    assert lines[0] == "%%MatrixMarket matrix coordinate real general"
    assert lines[1] == f"{A.m} {A.n} {A.nnz}"
    r0 = int(np.searchsorted(A.rowptr, 0, side="right")) - 1
    assert lines[2] == "%d %d %20.16g" % (r0 + 1, A.col[0] + 1, A.val[0])
    B, sym = load_mtx(p)
    assert not sym and np.array_equal(B.rowptr, A.rowptr) and np.array_equal(B.col, A.col)
    assert np.allclose(B.val, A.val, rtol=1e-15, atol=0)
    write_mtx(p, A, exact=True)
    B, _ = load_mtx(p)
    assert np.array_equal(B.val, A.val)


@pytest.fixture
def mtx_threads(monkeypatch):
    """Set TSG_MTX_THREADS for the loader (read at every call)."""
    def set_threads(n):
        monkeypatch.setenv("TSG_MTX_THREADS", str(n))
    return set_threads


@pytest.mark.parametrize("stem", FILES)
@pytest.mark.parametrize("threads", [1, 3, 8])
def test_threads_match_reference(built_lib, mtx_threads, stem, threads):
    """The line-parallel reader (tiny runs of lines here) and the token
    reader give the reference loader's result, or its refusal."""
    mtx_threads(threads)
    test_load_matches_reference(built_lib, stem)


def _load(path):
    from tilespgemm_gb300 import TSGError, load_mtx
    try:
        A, sym = load_mtx(path)
        return ("ok", A.m, A.n, int(sym), np.asarray(A.rowptr).tolist(), np.asarray(A.col).tolist(),
                np.asarray(A.val).view(np.int64).tolist())
    except TSGError as e:
        return ("err", e.status, str(e))


CASES = {
    "blank_lines_crlf": "%%MatrixMarket matrix coordinate real general\r\n4 4 3\r\n\r\n1 2 1.5\r\n  \r\n3 1 -2e-3\r\n4 4 7\r\n",
    "past_nz_ignored": "%%MatrixMarket matrix coordinate real general\n3 3 2\n1 1 1\n2 2 2\ngarbage here\n9 9 9\n",
    "split_entry": "%%MatrixMarket matrix coordinate real general\n3 3 2\n1 1\n1.0\n2 2 2.0\n",
    "extra_token": "%%MatrixMarket matrix coordinate real general\n3 3 2\n1 1 1.0 5\n2 2 2.0\n",
    "size_line_tail": "%%MatrixMarket matrix coordinate real general\n3 3 2 1 1 1.0\n2 2 2.0\n",
    "comment_in_data": "%%MatrixMarket matrix coordinate real general\n3 3 2\n1 1 1.0\n% note\n2 2 2.0\n",
    "truncated": "%%MatrixMarket matrix coordinate real general\n3 3 3\n1 1 1.0\n2 2 2.0\n",
    "truncated_value": "%%MatrixMarket matrix coordinate real general\n3 3 2\n1 1 1.0\n2 2\n",
    "outside": "%%MatrixMarket matrix coordinate real general\n3 3 3\n1 1 1.0\n4 2 2.0\n3 3 3.0\n",
    "outside_past_nz": "%%MatrixMarket matrix coordinate real general\n3 3 2\n1 1 1.0\n2 2 2.0\n4 4 4.0\n",
    "symmetric": "%%MatrixMarket matrix coordinate real symmetric\n4 4 5\n1 1 1\n3 1 2\n4 2 3\n2 1 4\n4 4 5\n",
    "integer": "%%MatrixMarket matrix coordinate integer general\n3 3 3\n1 1 3\n2 3 -4\n3 2 5000000000\n",
    "pattern": "%%MatrixMarket matrix coordinate pattern general\n3 3 3\n1 1\n2 3\n3 2\n",
    "complex": "%%MatrixMarket matrix coordinate complex hermitian\n3 3 2\n1 1 1.0 0.0\n3 1 2.5 -1.0\n",
    "no_final_newline": "%%MatrixMarket matrix coordinate real general\n2 2 2\n1 1 1.0\n2 2 2.0",
}


@pytest.mark.parametrize("name", list(CASES))
def test_threads_agree_on_edge_cases(built_lib, mtx_threads, tmp_path, name):
    """Line reader and token reader agree on blank lines, CRLF, lines past
    NZ, entries split over lines, extra tokens, comments and truncation."""
    p = tmp_path / f"{name}.mtx"
    p.write_bytes(CASES[name].encode())
    mtx_threads(1)
    want = _load(p)
    for t in (2, 3, 5, 16):
        mtx_threads(t)
        assert _load(p) == want, t


@pytest.mark.parametrize("sym", ["general", "symmetric"])
def test_threads_agree_on_a_large_file(built_lib, mtx_threads, tmp_path, sym):
    """~200,000 entries with random spacing: every thread count gives the
    token reader's CSR, bit for bit."""
    rng = np.random.default_rng(5)
    n, nz = 20000, 200000
    i = rng.integers(1, n + 1, nz)
    j = rng.integers(1, n + 1, nz)
    if sym == "symmetric":
        i, j = np.maximum(i, j), np.minimum(i, j)
    v = rng.standard_normal(nz) * 10.0 ** rng.integers(-5, 5, nz)
    sep = np.where(rng.random(nz) < 0.1, "  ", " ")
    lines = [f"{a}{s}{b} {x!r}" for a, b, x, s in zip(i.tolist(), j.tolist(), v.tolist(), sep.tolist())]
    p = tmp_path / "big.mtx"
    p.write_text(f"%%MatrixMarket matrix coordinate real {sym}\n% generated\n{n} {n} {nz}\n" + "\n".join(lines) + "\n")
    mtx_threads(1)
    want = _load(p)
    assert want[0] == "ok"
    for t in (2, 7, 32):
        mtx_threads(t)
        assert _load(p) == want, t


@pytest.mark.parametrize("exact", [False, True])
def test_writer_threads_write_the_same_bytes(built_lib, mtx_threads, tmp_path, exact):
    """tsg_write_mtx formats waves of rows on several threads: the file is
    byte for byte the one-thread file (empty rows, a long row, int64 row
    pointers), and it loads back."""
    from tilespgemm_gb300 import load_mtx, write_mtx
    from tilespgemm_gb300 import matrices as M
    from tilespgemm_gb300.api import CSR
    A = M.random_sparse(3000, 2500, 9, seed=12, empty_rows=0.2)
    rp = np.asarray(A.rowptr, np.int64)
    long_row = np.arange(0, 2500, 2, dtype=np.int32)             # row 7 gets 1,250 entries
    cols = [np.asarray(A.col[rp[r]:rp[r + 1]]) for r in range(A.m)]
    vals = [np.asarray(A.val[rp[r]:rp[r + 1]]) for r in range(A.m)]
    cols[7], vals[7] = long_row, np.linspace(-3.0, 3.0, long_row.size)
    rp2 = np.concatenate([[0], np.cumsum([c.size for c in cols])]).astype(np.int64)
    B = CSR(A.m, A.n, rp2, np.concatenate(cols), np.concatenate(vals))
    for X in (A, B):
        mtx_threads(1)
        write_mtx(tmp_path / "one.mtx", X, exact=exact)
        want = (tmp_path / "one.mtx").read_bytes()
        for t in (2, 5, 16):
            mtx_threads(t)
            write_mtx(tmp_path / "many.mtx", X, exact=exact)
            assert (tmp_path / "many.mtx").read_bytes() == want, t
        Y, _ = load_mtx(tmp_path / "many.mtx")
        assert np.array_equal(np.asarray(Y.rowptr, np.int64), np.asarray(X.rowptr, np.int64))
        assert np.array_equal(Y.col, X.col)
        if exact:
            assert np.array_equal(Y.val, X.val)


def test_writer_refuses_a_bad_row_pointer(built_lib, tmp_path):
    from tilespgemm_gb300 import TSGError, write_mtx
    from tilespgemm_gb300.api import CSR
    X = CSR(3, 3, np.array([0, 2, 1, 3], np.int64), np.array([0, 1, 2], np.int32), np.ones(3))
    with pytest.raises(TSGError):
        write_mtx(tmp_path / "bad.mtx", X)


def test_writer_waves(built_lib, mtx_threads, tmp_path):
    """More entries than one wave (2^20 per thread): several waves, written
    in order, give the one-thread bytes."""
    from tilespgemm_gb300 import write_mtx
    from tilespgemm_gb300 import matrices as M
    A = M.random_sparse(150000, 150000, 16, seed=4)     # 2.4 M entries: three waves on one thread, two on two
    assert A.nnz > 2 * (1 << 20)
    mtx_threads(1)
    write_mtx(tmp_path / "one.mtx", A)
    mtx_threads(2)
    write_mtx(tmp_path / "two.mtx", A)
    assert (tmp_path / "one.mtx").read_bytes() == (tmp_path / "two.mtx").read_bytes()
