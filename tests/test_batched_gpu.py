"""Batched products (tsg_spgemm_batched): every instance of one block-diagonal
pass equals its own single product, bit for bit."""
import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu


def _instances(count, seed, square=True):
    from tilespgemm_gb300 import matrices as M
    rng = np.random.default_rng(seed)
    out = []
    for i in range(count):
        n = int(np.exp(rng.uniform(np.log(5), np.log(700))))
        k = n if square else int(np.exp(rng.uniform(np.log(5), np.log(700))))
        nnz_row = int(rng.integers(1, 12))
        band = max(1, n // 8) if i % 2 == 0 else None
        out.append(M.random_sparse(n, k, nnz_row, seed=seed * 1000 + i, band=band))
    return out


def _check(C, A, B):
    rp, col, val = O.spgemm(A, B)
    assert C.m == A.m and C.n == B.n
    assert np.array_equal(np.asarray(C.rowptr, np.int64), rp)
    assert np.array_equal(C.col, col)
    assert np.array_equal(C.val, val)


def test_batched_aa_host(ctx):
    As = _instances(40, 1)
    Cs = ctx.spgemm_batched(As, op="AA")
    for A, C in zip(As, Cs):
        _check(C, A, A)


def test_batched_aat_and_device(ctx):
    from tilespgemm_gb300.api import CSR
    As = _instances(25, 2, square=False)
    outs, st = ctx.spgemm_batched_raw([A.to_device(0) for A in As], op="AAT", out="device", stats=True)
    assert st["nnz_c"] == sum(o.nnz for o in outs)
    for A, oc in zip(As, outs):
        C = oc.download()
        tp, tr, tv = O.transpose(A)
        _check(C, A, CSR(A.n, A.m, tp, tr, tv))
    for oc in outs:
        oc.free()


def test_batched_ab_and_edge_instances(ctx):
    from tilespgemm_gb300 import matrices as M
    from tilespgemm_gb300.api import CSR
    As = [M.random_sparse(33, 50, 4, seed=3), CSR(0, 7, np.zeros(1, np.int64), np.zeros(0, np.int32), np.zeros(0)),
          M.random_sparse(16, 16, 3, seed=4), CSR(5, 9, np.zeros(6, np.int64), np.zeros(0, np.int32), np.zeros(0))]
    Bs = [M.random_sparse(50, 21, 5, seed=5), M.random_sparse(7, 3, 2, seed=6),
          M.random_sparse(16, 40, 3, seed=7), M.random_sparse(9, 12, 2, seed=8)]
    Cs = ctx.spgemm_batched(As, Bs, op="AB")
    for A, B, C in zip(As, Bs, Cs):
        _check(C, A, B)


def test_batched_matches_one_at_a_time(ctx):
    As = _instances(12, 9)
    Cs = ctx.spgemm_batched(As, op="AA")
    for A, C in zip(As, Cs):
        D = ctx.spgemm(A, op="AA")
        assert np.array_equal(C.col, D.col) and np.array_equal(C.val, D.val)


def test_batched_bad_instance_is_reported(ctx):
    from tilespgemm_gb300 import TSGError
    from tilespgemm_gb300.api import CSR
    good = CSR(3, 3, np.array([0, 1, 2, 3]), np.array([0, 1, 2], np.int32), np.ones(3))
    bad = CSR(3, 3, np.array([0, 1, 2, 3]), np.array([0, 7, 2], np.int32), np.ones(3))
    with pytest.raises(TSGError) as e:
        ctx.spgemm_batched([good, bad], op="AA")
    assert e.value.status == 8


def test_sibling_results_freed_from_many_threads(ctx):
    """The results of one batched call share one allocation that goes with
    the last of them.  Freed from eight threads at once, it is released
    exactly once: results of later calls get buffers of their own (a buffer
    released twice would be handed to two live results) and stay exact."""
    import threading
    As = _instances(64, 21)
    for _ in range(4):
        outs, _ = ctx.spgemm_batched_raw(As, op="AA", out="host")
        gate = threading.Barrier(8)

        def work(part):
            gate.wait()
            for o in part:
                o.free()

        ths = [threading.Thread(target=work, args=(outs[t::8],)) for t in range(8)]
        for t in ths:
            t.start()
        for t in ths:
            t.join()
        assert all(not o.s.owner for o in outs)
    first, _ = ctx.spgemm_batched_raw(As[:32], op="AA", out="host")
    second, _ = ctx.spgemm_batched_raw(As[32:], op="AA", out="host")
    try:
        for A, oc in zip(As, first + second):
            _check(oc.download(), A, A)
    finally:
        for oc in first + second:
            oc.free()
