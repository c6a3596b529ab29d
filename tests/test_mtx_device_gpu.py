"""Device-side Matrix Market parsing (tsg_load_mtx_device) against the host
loader (tsg_load_mtx) and the reference loader's outputs (mtx_*.npz): the
same CSR entry for entry -- row pointers, columns in file order per row,
mirrored entries after their sources, values bit for bit -- and the same
errors."""
import numpy as np
import pytest

from conftest import GOLDEN

pytestmark = pytest.mark.gpu
FILES = sorted(p.stem for p in (GOLDEN / "mtx").glob("*.mtx"))


def _dev_load(ctx, path):
    oc, sym = ctx.load_mtx_device(path)
    try:
        assert oc.where == "device" and oc.rowptr_bits == 32
        return oc.download(), sym
    finally:
        oc.free()


def _same(A, B):
    assert (A.m, A.n, A.nnz) == (B.m, B.n, B.nnz)
    assert np.array_equal(np.asarray(A.rowptr, np.int64), np.asarray(B.rowptr, np.int64))
    assert np.array_equal(A.col, B.col)
    assert np.array_equal(A.val.view(np.int64), B.val.view(np.int64))   # bit for bit, signed zeros included


@pytest.mark.parametrize("stem", FILES)
def test_device_load_matches_reference(ctx, stem):
    from tilespgemm_gb300 import TSGError, load_mtx
    g = np.load(GOLDEN / f"mtx_{stem}.npz")
    path = GOLDEN / "mtx" / f"{stem}.mtx"
    if int(g["rc"]) != 0:
        with pytest.raises(TSGError) as ei:
            _dev_load(ctx, path)
        assert ei.value.status == 5
        return
    A, sym = _dev_load(ctx, path)
    assert (A.m, A.n, A.nnz, int(sym)) == (int(g["m"]), int(g["n"]), int(g["nnz"]), int(g["sym"]))
    assert np.array_equal(np.asarray(A.rowptr, np.int64), g["rowptr"].astype(np.int64))
    assert np.array_equal(A.col, g["col"])
    assert np.array_equal(A.val, g["val"])
    H, hsym = load_mtx(path)
    _same(A, H)


def _write(path, banner, m, n, lines):
    with open(path, "w") as f:
        f.write(banner + "\n% generated\n")
        f.write(f"{m} {n} {len([x for x in lines if x.strip()])}\n")
        for x in lines:
            f.write(x + "\n")


@pytest.mark.parametrize("sym", ["general", "symmetric", "skew-symmetric"])
def test_device_load_generated_formats(ctx, tmp_path, sym):
    """A larger file (many 4 KB chunks) with every value format the reader
    meets: short decimals (parsed on the device), 17-digit values, large and
    small exponents, signed zeros, '+' signs, hex and inf (left to the
    host), blank lines, tabs and carriage returns."""
    from tilespgemm_gb300 import load_mtx
    rng = np.random.default_rng(5)
    m = n = 3000
    out = []
    seen = set()
    while len(seen) < 40000:
        i, j = int(rng.integers(1, m + 1)), int(rng.integers(1, n + 1))
        if sym != "general" and j > i:
            i, j = j, i
        if sym == "skew-symmetric" and i == j:
            continue
        if (i, j) in seen and rng.random() < 0.9:
            continue
        seen.add((i, j))
        k = len(seen) % 12
        v = rng.uniform(-10, 10)
        s = {0: f"{v:.3f}", 1: f"{v!r}", 2: f"{v:.17g}", 3: f"{v:.6e}", 4: f"{v * 1e-30:.5e}", 5: f"{v * 1e25:.4e}",
             6: "-0.0", 7: f"+{abs(v):.2f}", 8: float(v).hex(), 9: "inf" if rng.random() < 0.5 else "-inf",
             10: f"{int(v)}", 11: f"{v:.1f}e+2"}[k]
        sep = "\t" if k % 3 == 0 else " "
        line = f"{i}{sep}{j} {s}" + ("\r" if k == 4 else "")
        out.append(line)
        if k == 5:
            out.append("   ")
    path = tmp_path / "g.mtx"
    _write(path, f"%%MatrixMarket matrix coordinate real {sym}", m, n, out)
    H, hsym = load_mtx(path)
    A, dsym = _dev_load(ctx, path)
    assert hsym == dsym
    _same(A, H)


@pytest.mark.parametrize("kind", ["integer", "pattern", "complex"])
def test_device_load_value_kinds(ctx, tmp_path, kind):
    from tilespgemm_gb300 import load_mtx
    rng = np.random.default_rng(6)
    lines = []
    for t in range(5000):
        i, j = int(rng.integers(1, 801)), int(rng.integers(1, 701))
        if kind == "integer":
            lines.append(f"{i} {j} {int(rng.integers(-5_000_000_000, 5_000_000_000))}")
        elif kind == "pattern":
            lines.append(f"{i} {j}")
        else:
            lines.append(f"{i} {j} {rng.uniform(-1, 1):.4f} {rng.uniform(-1, 1):.17g}")
    path = tmp_path / "k.mtx"
    _write(path, f"%%MatrixMarket matrix coordinate {kind} hermitian" if kind == "complex" else
           f"%%MatrixMarket matrix coordinate {kind} general", 800, 800 if kind == "complex" else 700, lines)
    H, _ = load_mtx(path)
    A, _ = _dev_load(ctx, path)
    _same(A, H)


def test_device_load_errors_and_fallback(ctx, tmp_path):
    """The host loader's statuses; an entry split over two lines (read token
    by token by the host loader) gives the host loader's matrix."""
    from tilespgemm_gb300 import TSGError, load_mtx
    p = tmp_path / "e.mtx"
    cases = [
        "%%MatrixMarket matrix coordinate real general\n3 3 2\n1 1 1.0\n",            # truncated
        "%%MatrixMarket matrix coordinate real general\n3 3 1\n4 1 1.0\n",            # outside
        "%%MatrixMarket matrix coordinate real general\n3 3 1\n1 1 0x1p400000\n",     # outside the double range: host reads it
        "%%MatrixMarket matrix coordinate real symmetric\n2 3 1\n1 3 1.0\n",           # mirror outside
        "%%MatrixMarket matrix array real general\n2 2\n1\n2\n3\n4\n",                 # array
    ]
    for text in cases:
        p.write_text(text)
        try:
            H, _ = load_mtx(p)
            host = None
        except TSGError as e:
            host = e.status
        if host is None:
            A, _ = _dev_load(ctx, p)
            _same(A, H)
        else:
            with pytest.raises(TSGError) as ei:
                _dev_load(ctx, p)
            assert ei.value.status == host
    p.write_text("%%MatrixMarket matrix coordinate real general\n3 3 3\n1 1\n1.5\n2 2 2.5\n3 3 3.5\n")
    H, _ = load_mtx(p)
    A, _ = _dev_load(ctx, p)
    _same(A, H)
    with pytest.raises(TSGError) as ei:
        _dev_load(ctx, tmp_path / "missing.mtx")
    assert ei.value.status == 5
