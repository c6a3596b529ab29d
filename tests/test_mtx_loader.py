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
