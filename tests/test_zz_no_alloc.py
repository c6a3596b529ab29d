"""tsg_tiles_to_csr_noalloc against tsg_tiles_to_csr (the allocating entry
point): two calls in a row into caller buffers, bit-exact, plus the row
limit.  The file name keeps it last in collection, so it also runs after
every other GPU test has used the library."""
import ctypes as C

import numpy as np
import pytest

from tilespgemm_gb300 import _abi, matrices as M

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    from tilespgemm_gb300 import Context
    c = Context(0)
    yield c
    c.close()


def _tiles(ctx, A):
    """Device tile form of A from the existing conversion (allocates; set-up)."""
    a, keep = A._tsg()
    t = _abi.tsg_tiles()
    _abi.check(_abi.lib().tsg_csr_to_tiles(ctx.handle, C.byref(a), C.byref(t)))
    del keep
    return t


def _existing(ctx, t):
    c = _abi.tsg_csr()
    _abi.check(_abi.lib().tsg_tiles_to_csr(ctx.handle, C.byref(t), C.byref(c)))
    rp = np.empty(c.m + 1, np.int64)
    col = np.empty(c.nnz, np.int32)
    val = np.empty(c.nnz, np.float64)
    _abi.check(_abi.lib().tsg_csr_download(ctx.handle, C.byref(c), rp.ctypes.data,
                                           col.ctypes.data if c.nnz else None, val.ctypes.data if c.nnz else None))
    _abi.lib().tsg_csr_free(ctx.handle, C.byref(c))
    return rp, col, val


def _noalloc(ctx, t, bufs):
    rp_d, col_d, val_d = bufs
    _abi.check(_abi.lib().tsg_tiles_to_csr_noalloc(ctx.handle, C.byref(t), rp_d.data_ptr(),
                                                   col_d.data_ptr() if t.nnz else None,
                                                   val_d.data_ptr() if t.nnz else None))
    n = int(t.nnz)
    return rp_d.cpu().numpy(), col_d[:n].cpu().numpy(), val_d[:n].cpu().numpy()


def test_two_calls_in_a_row_match_existing(ctx):
    import torch
    mats = [M.random_sparse(3001, 2777, 9, seed=11, empty_rows=0.1),
            M.rmat(11, 8, seed=7)]
    # caller buffers sized once for the larger case and reused by both calls
    m_max = max(A.m for A in mats)
    nnz_max = max(A.nnz for A in mats)
    dev = torch.device("cuda", 0)
    bufs = (torch.full((m_max + 1,), -7, dtype=torch.int64, device=dev),
            torch.full((nnz_max,), -7, dtype=torch.int32, device=dev),
            torch.full((nnz_max,), float("nan"), dtype=torch.float64, device=dev))
    for A in mats:
        t = _tiles(ctx, A)
        try:
            rp0, col0, val0 = _existing(ctx, t)
            views = (bufs[0][:A.m + 1], bufs[1], bufs[2])
            rp1, col1, val1 = _noalloc(ctx, t, views)
        finally:
            _abi.lib().tsg_tiles_free(ctx.handle, C.byref(t))
        np.testing.assert_array_equal(rp1, rp0)
        np.testing.assert_array_equal(col1, col0)
        assert np.array_equal(val1.view(np.int64), val0.view(np.int64))
        # and both are A itself
        np.testing.assert_array_equal(rp1, np.asarray(A.rowptr, np.int64))
        np.testing.assert_array_equal(col1, np.asarray(A.col))
        assert np.array_equal(val1, np.asarray(A.val))


def test_empty_and_row_limit(ctx):
    import torch
    dev = torch.device("cuda", 0)
    A = M.random_sparse(40, 40, 3, seed=2, empty_rows=1.0)   # no entries at all
    t = _tiles(ctx, A)
    try:
        rp = torch.full((A.m + 1,), -1, dtype=torch.int64, device=dev)
        _abi.check(_abi.lib().tsg_tiles_to_csr_noalloc(ctx.handle, C.byref(t), rp.data_ptr(), None, None))
        assert rp.cpu().numpy().tolist() == [0] * (A.m + 1)
        # more rows than the static scratch holds: refused before any device work
        big = _abi.tsg_tiles()
        C.memmove(C.byref(big), C.byref(t), C.sizeof(_abi.tsg_tiles))
        big.m = _abi.NOALLOC_MAX_ROWS + 1
        big.blkm = (big.m + 15) // 16
        st = _abi.lib().tsg_tiles_to_csr_noalloc(ctx.handle, C.byref(big), rp.data_ptr(), None, None)
        assert st == _abi.ERR_NOT_SUPPORTED
        assert b"TSG_NOALLOC_MAX_ROWS" in _abi.lib().tsg_last_error()
    finally:
        _abi.lib().tsg_tiles_free(ctx.handle, C.byref(t))


def test_refuses_buffers_off_the_device(ctx):
    """Outputs must be memory the context's GPU writes: pinned host memory,
    and device memory of another GPU where there is one, are refused with
    TSG_ERR_INVALID_ARG before any device work."""
    import torch
    A = M.random_sparse(300, 300, 4, seed=5)
    t = _tiles(ctx, A)
    try:
        dev = torch.device("cuda", 0)
        rp_h = torch.zeros(A.m + 1, dtype=torch.int64).pin_memory()
        col = torch.empty(A.nnz, dtype=torch.int32, device=dev)
        val = torch.empty(A.nnz, dtype=torch.float64, device=dev)
        st = _abi.lib().tsg_tiles_to_csr_noalloc(ctx.handle, C.byref(t), rp_h.data_ptr(), col.data_ptr(),
                                                 val.data_ptr())
        assert st == _abi.ERR_INVALID_ARG
        assert rp_h.numpy().tolist() == [0] * (A.m + 1)
        if torch.cuda.device_count() > 1:
            other = torch.device("cuda", 1)
            rp_o = torch.zeros(A.m + 1, dtype=torch.int64, device=other)
            st = _abi.lib().tsg_tiles_to_csr_noalloc(ctx.handle, C.byref(t), rp_o.data_ptr(), col.data_ptr(),
                                                     val.data_ptr())
            assert st == _abi.ERR_INVALID_ARG
    finally:
        _abi.lib().tsg_tiles_free(ctx.handle, C.byref(t))
