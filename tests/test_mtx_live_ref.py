"""The host Matrix Market loader (tsg_load_mtx) and writer (tsg_write_mtx)
against the reference's own mmio_allinone (mmio_highlevel.h:593-759) and
mm_write_mtx_crd (mmio.h:780-850), called live on generated files.

These are well-formed files of every value type and symmetry the loader
takes.  Entries are in random order, with duplicates, explicit zeros,
varied number formats and spacing, CRLF line ends and blank lines.  The
loader's result must equal the reference's entry for entry, with one and
with several parsing threads.

This needs the reference's CPU code built into oracle/_ref (by
oracle/build_ref.sh from a reference checkout on this machine); without it
the module is skipped, and the committed fixtures pin the loader
(test_mtx_loader.py).  Only well-formed files are given to the reference,
which does not check indices against the size line.
"""
import ctypes as C
import zlib

import numpy as np
import pytest

from conftest import ROOT

REF = ROOT / "oracle" / "_ref"


@pytest.fixture(scope="module")
def ref_loader():
    try:
        st = C.CDLL(str(REF / "libstir_ref.so"))
    except OSError as e:
        pytest.skip(f"the reference's CPU code is not built here ({e})")
    IP, DP = C.POINTER(C.c_int), C.POINTER(C.c_double)

    def load(path):
        m, n, nnz, sym = C.c_int(0), C.c_int(0), C.c_int(0), C.c_int(0)
        rp, col, val = IP(), IP(), DP()
        rc = st.ref_mmio_allinone(C.byref(m), C.byref(n), C.byref(nnz), C.byref(sym), C.byref(rp), C.byref(col),
                                  C.byref(val), str(path).encode())
        assert rc == 0, f"the reference refused a well-formed file ({rc})"
        rpa = np.ctypeslib.as_array(rp, shape=(m.value + 1,)).copy()
        cola = np.ctypeslib.as_array(col, shape=(max(nnz.value, 1),))[:nnz.value].copy()
        vala = np.ctypeslib.as_array(val, shape=(max(nnz.value, 1),))[:nnz.value].copy()
        return m.value, n.value, sym.value, rpa, cola, vala
    return load


def _fmt(rng, x: float) -> str:
    k = int(rng.integers(0, 5))
    if k == 0:
        return repr(float(x))
    if k == 1:
        return f"{x:.3e}"
    if k == 2:
        return f"{x:.17g}"
    if k == 3:
        return f"{x:.6f}"
    return f"{x:.2E}"


def _write(path, rng, kind: str, sym: str, m: int, n: int, nz: int, crlf: bool):
    i = rng.integers(1, m + 1, nz)
    j = rng.integers(1, n + 1, nz)
    if sym != "general":
        i, j = np.maximum(i, j), np.minimum(i, j)
        if sym == "skew-symmetric":   # no diagonal entries in a skew-symmetric file
            keep = i != j
            i, j = i[keep], j[keep]
    if nz > 4:                        # a duplicate entry
        i[-1], j[-1] = i[0], j[0]
    nz = int(i.size)
    v = rng.standard_normal(nz) * 10.0 ** rng.integers(-4, 4, nz)
    v[rng.random(nz) < 0.05] = 0.0    # explicit zeros
    lines = []
    for a, b, x in zip(i.tolist(), j.tolist(), v.tolist()):
        sp = " " if rng.random() < 0.8 else "   "
        if kind == "real":
            lines.append(f"{a}{sp}{b} {_fmt(rng, x)}")
        elif kind == "integer":
            lines.append(f"{a}{sp}{b} {int(round(x * 100)) % 100000 - 50000}")
        elif kind == "complex":
            lines.append(f"{a}{sp}{b} {_fmt(rng, x)} {_fmt(rng, -x / 3)}")
        else:
            lines.append(f"{a}{sp}{b}")
        if rng.random() < 0.02:
            lines.append("")          # a blank line between entries
    nl = "\r\n" if crlf else "\n"
    text = nl.join([f"%%MatrixMarket matrix coordinate {kind} {sym}", "% generated", f"{m} {n} {nz}"] + lines) + nl
    path.write_bytes(text.encode())


FILES = []
for kind, syms in (("real", ("general", "symmetric", "skew-symmetric")), ("integer", ("general", "symmetric")),
                   ("pattern", ("general", "symmetric")), ("complex", ("general", "hermitian", "symmetric"))):
    for sym in syms:
        FILES.append((kind, sym))


@pytest.mark.parametrize("crlf", [False, True])
@pytest.mark.parametrize("kind,sym", FILES, ids=[f"{k}-{s}" for k, s in FILES])
def test_loader_matches_reference_live(built_lib, ref_loader, monkeypatch, tmp_path, kind, sym, crlf):
    from tilespgemm_gb300 import load_mtx
    rng = np.random.default_rng(zlib.crc32(f"{kind}/{sym}/{crlf}".encode()))
    square = sym != "general"
    for t, (m, n, nz) in enumerate([(37, 37 if square else 51, 120), (400, 400 if square else 300, 6000)]):
        p = tmp_path / f"f{t}.mtx"
        _write(p, rng, kind, sym, m, n, nz, crlf)
        rm, rn, rsym, rrp, rcol, rval = ref_loader(p)
        for threads in (1, 8):
            monkeypatch.setenv("TSG_MTX_THREADS", str(threads))
            A, s = load_mtx(p)
            assert (A.m, A.n, int(s)) == (rm, rn, rsym)
            assert np.array_equal(np.asarray(A.rowptr, np.int64), rrp.astype(np.int64))
            assert np.array_equal(np.asarray(A.col), rcol)
            assert np.array_equal(np.asarray(A.val).view(np.int64), rval.view(np.int64))


@pytest.fixture(scope="module")
def ref_writer():
    try:
        st = C.CDLL(str(REF / "libstir_ref.so"))
        f = st.ref_mm_write_mtx_crd
    except (OSError, AttributeError) as e:
        pytest.skip(f"the reference's writer is not built here ({e})")
    f.restype = C.c_int

    def write(path, A):
        rp = np.asarray(A.rowptr, np.int64)
        rows = np.repeat(np.arange(A.m, dtype=np.int32), np.diff(rp).astype(np.int64)) + 1
        cols = np.ascontiguousarray(np.asarray(A.col, np.int32) + 1)
        vals = np.ascontiguousarray(np.asarray(A.val, np.float64))
        rc = f(str(path).encode(), A.m, A.n, int(A.nnz), rows.ctypes.data_as(C.c_void_p),
               cols.ctypes.data_as(C.c_void_p), vals.ctypes.data_as(C.c_void_p))
        assert rc == 0
    return write


@pytest.mark.parametrize("threads", [1, 8])
def test_writer_matches_reference_live(built_lib, ref_writer, monkeypatch, tmp_path, threads):
    """tsg_write_mtx (the reference's line format) gives the bytes of the
    reference's mm_write_mtx_crd for the same entries in CSR order: varied
    magnitudes, negative zeros, duplicate and unsorted columns, empty rows."""
    from tilespgemm_gb300 import matrices as M
    from tilespgemm_gb300 import write_mtx
    from tilespgemm_gb300.api import CSR
    monkeypatch.setenv("TSG_MTX_THREADS", str(threads))
    rng = np.random.default_rng(77)
    for t, (m, n, k) in enumerate([(1, 1, 1), (53, 41, 3), (700, 900, 9)]):
        X = M.random_sparse(m, n, k, seed=200 + t, dup=True, unsorted=True, empty_rows=0.2)
        v = rng.standard_normal(X.nnz) * 10.0 ** rng.integers(-300, 300, X.nnz)
        v[rng.random(X.nnz) < 0.05] = -0.0
        A = CSR(X.m, X.n, np.asarray(X.rowptr, np.int64), np.asarray(X.col, np.int32), v)
        ours, theirs = tmp_path / f"ours{t}.mtx", tmp_path / f"ref{t}.mtx"
        write_mtx(ours, A)
        ref_writer(theirs, A)
        assert ours.read_bytes() == theirs.read_bytes()
