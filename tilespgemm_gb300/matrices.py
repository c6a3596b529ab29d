"""Seeded synthetic operands with the shapes and value distributions of the
workloads this library is measured on (the reference's SuiteSparse inputs
are not available, so these generators stand in for them).

All generators return host CSR (numpy) with int32 column indices sorted
within each row and FP64 values; random streams use numpy's Philox
(counter-based) generator.
"""
from __future__ import annotations

import numpy as np

from .api import CSR


def _rng(seed: int) -> np.random.Generator:
    return np.random.Generator(np.random.Philox(seed))


def _from_coo(m: int, n: int, r: np.ndarray, c: np.ndarray, v: np.ndarray, merge: bool) -> CSR:
    """COO -> CSR with columns sorted per row; duplicates summed when `merge`."""
    key = r.astype(np.int64) * n + c.astype(np.int64)
    order = np.argsort(key, kind="stable")
    key, v = key[order], v[order]
    if merge and key.size:
        first = np.ones(key.size, dtype=bool)
        first[1:] = key[1:] != key[:-1]
        idx = np.cumsum(first) - 1
        vsum = np.zeros(int(first.sum()), dtype=np.float64)
        np.add.at(vsum, idx, v)
        key, v = key[first], vsum
    rows = (key // n).astype(np.int64)
    cols = (key % n).astype(np.int32)
    rp = np.zeros(m + 1, dtype=np.int64)
    np.add.at(rp, rows + 1, 1)
    rp = np.cumsum(rp)
    return CSR(m, n, rp, cols, v.astype(np.float64))


def laplacian_2d(nx: int, ny: int | None = None) -> CSR:
    """5-point Laplacian on an nx*ny grid, natural row-major ordering,
    diagonal 4.0 and off-diagonals -1.0 (the 256x256 case has 326,656 nnz)."""
    ny = nx if ny is None else ny
    n = nx * ny
    idx = np.arange(n, dtype=np.int64)
    x, y = idx % nx, idx // nx
    rs, cs, vs = [idx], [idx], [np.full(n, 4.0)]
    for dx, dy in ((-1, 0), (1, 0), (0, -1), (0, 1)):
        ok = (x + dx >= 0) & (x + dx < nx) & (y + dy >= 0) & (y + dy < ny)
        rs.append(idx[ok])
        cs.append(idx[ok] + dx + dy * nx)
        vs.append(np.full(int(ok.sum()), -1.0))
    return _from_coo(n, n, np.concatenate(rs), np.concatenate(cs), np.concatenate(vs), merge=False)


def stencil_27(side: int, seed: int = 1) -> CSR:
    """27-point stencil on a side^3 grid, natural ordering, off-diagonal values
    uniform in [0.5, 1.5], diagonal = sum of the row's off-diagonals
    (side 96: n = 884,736, 23,393,656 nnz)."""
    n = side ** 3
    idx = np.arange(n, dtype=np.int64)
    x, y, z = idx % side, (idx // side) % side, idx // (side * side)
    rows, cols = [], []
    for dz in (-1, 0, 1):
        for dy in (-1, 0, 1):
            for dx in (-1, 0, 1):
                ok = ((x + dx >= 0) & (x + dx < side) & (y + dy >= 0) & (y + dy < side)
                      & (z + dz >= 0) & (z + dz < side))
                rows.append(idx[ok])
                cols.append(idx[ok] + dx + dy * side + dz * side * side)
    r = np.concatenate(rows)
    c = np.concatenate(cols)
    A = _from_coo(n, n, r, c, np.zeros(r.size), merge=False)
    rng = _rng(seed)
    val = rng.uniform(0.5, 1.5, size=A.nnz)
    rowid = np.repeat(np.arange(n, dtype=np.int64), np.diff(A.rowptr))
    diag = A.col.astype(np.int64) == rowid
    val[diag] = 0.0
    rowsum = np.add.reduceat(val, A.rowptr[:-1]) if n else val
    val[diag] = rowsum[rowid[diag]]
    A.val = val
    return A


def rmat(scale: int, edge_factor: int = 16, abcd=(0.57, 0.19, 0.19, 0.05), seed: int = 1) -> CSR:
    """R-MAT graph with 2^scale vertices and edge_factor * 2^scale edges drawn;
    duplicates merged, self-loops kept, values uniform in [-1, 1]."""
    n = 1 << scale
    ne = edge_factor * n
    rng = _rng(seed)
    a, b, c, _ = abcd
    r = np.zeros(ne, dtype=np.int64)
    cc = np.zeros(ne, dtype=np.int64)
    for lvl in range(scale):
        u = rng.random(ne)
        right = (u >= a) & (u < a + b) | (u >= a + b + c)
        down = u >= a + b
        r |= down.astype(np.int64) << (scale - 1 - lvl)
        cc |= right.astype(np.int64) << (scale - 1 - lvl)
    A = _from_coo(n, n, r, cc, np.zeros(ne), merge=True)
    A.val = rng.uniform(-1.0, 1.0, size=A.nnz)
    return A


def random_sparse(m: int, n: int, nnz_per_row: int, seed: int = 0, band: int | None = None,
                  dup: bool = False, unsorted: bool = False, empty_rows: float = 0.0) -> CSR:
    """Uniform (or banded, |i-j| <= band) random sparse matrix for tests.
    dup keeps duplicate entries, unsorted shuffles columns inside rows,
    empty_rows is the fraction of rows left empty."""
    rng = _rng(seed)
    r = np.repeat(np.arange(m, dtype=np.int64), nnz_per_row)
    if band is None:
        c = rng.integers(0, n, size=r.size)
    else:
        c = np.clip(r + rng.integers(-band, band + 1, size=r.size), 0, n - 1)
    if empty_rows > 0:
        keep = rng.random(m) >= empty_rows
        sel = keep[r]
        r, c = r[sel], c[sel]
    v = rng.uniform(-1.0, 1.0, size=r.size)
    A = _from_coo(m, n, r, c, v, merge=not dup)
    if unsorted and A.nnz:
        perm = np.arange(A.nnz)
        for i in range(m):
            s, e = A.rowptr[i], A.rowptr[i + 1]
            if e - s > 1:
                perm[s:e] = s + rng.permutation(e - s)
        A.col, A.val = A.col[perm], A.val[perm]
    return A


def ref_values(A: CSR) -> CSR:
    """The reference's value convention val[i] = i % 10 (main_spgemm-col.cu:4895-4896):
    small integers, so every FP64 sum is exact in any order."""
    return CSR(A.m, A.n, A.rowptr, A.col, (np.arange(A.nnz) % 10).astype(np.float64))


def transpose(A: CSR) -> CSR:
    import scipy.sparse as sp
    s = sp.csr_matrix((A.val, A.col, A.rowptr), shape=(A.m, A.n)).T.tocsr()
    return CSR.from_scipy(s)


def batch_instance(i: int, seed: int = 1, n_range=(64, 16384), nnz_range=(2, 64)) -> CSR:
    """Instance i of the batched workload: n log-uniform in n_range, nnz/row
    uniform in nnz_range (drawn once per instance), columns banded
    (|i-j| <= n/16, bandwidth n/8) for even i and uniform for odd i,
    duplicates merged, values uniform in [-1, 1]."""
    rng = _rng(seed * 1_000_003 + i)
    n = int(round(np.exp(rng.uniform(np.log(n_range[0]), np.log(n_range[1])))))
    k = int(rng.integers(nnz_range[0], nnz_range[1] + 1))
    k = min(k, n)
    rows = np.arange(n, dtype=np.int64)[:, None]
    if i % 2 == 0:
        half = max(1, n // 16)
        lo = np.maximum(rows - half, 0)
        hi = np.minimum(rows + half, n - 1)
        cols = lo + np.floor(rng.random((n, k)) * (hi - lo + 1)).astype(np.int64)
    else:
        cols = rng.integers(0, n, size=(n, k))
    cols.sort(axis=1)
    keep = np.ones_like(cols, dtype=bool)
    keep[:, 1:] = cols[:, 1:] != cols[:, :-1]
    counts = keep.sum(axis=1)
    rp = np.zeros(n + 1, dtype=np.int64)
    np.cumsum(counts, out=rp[1:])
    col = cols[keep].astype(np.int32)
    val = rng.uniform(-1.0, 1.0, size=col.size)
    return CSR(n, n, rp, col, val)
