"""Failure detection without a GPU fault.

* A bounded device wait that runs out: the library's look-back scan is run
  with its first tile never published (tsg_check_bounded_wait); the waits
  give up after a short limit, the kernel finishes, the call returns
  TSG_ERR_DEVICE_TIMEOUT and the context keeps working.
* Allocation failures injected on the host (tsg_inject_alloc_failure): the
  k-th device-pool allocation of a call fails, for every k the call makes,
  and likewise pinned host memory for host results.  Each failed call
  returns TSG_ERR_OOM and the next call on the same context is exact.
The reference has neither: its look-back spins without bound
(utils_cuda_scan.h:167-170) and it checks no allocation.
"""
import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu


@pytest.fixture()
def fresh():
    from tilespgemm_gb300 import Context, _abi
    c = Context(0, small_path=0)
    yield c
    _abi.lib().tsg_inject_alloc_failure(0, 0)
    _abi.lib().tsg_inject_alloc_failure(1, 0)
    c.close()


def _exact(ctx, A, op):
    from tilespgemm_gb300.api import CSR
    C = ctx.spgemm(A, op=op)
    B = A
    if op == "AAT":
        tp, tr, tv = O.transpose(A)
        B = CSR(A.n, A.m, tp, tr, tv)
    rp, col, val = O.spgemm(A, B)
    assert np.array_equal(np.asarray(C.rowptr, np.int64), rp)
    assert np.array_equal(C.col, col)
    assert np.array_equal(C.val, val)


def test_bounded_wait_gives_up_and_context_survives(fresh):
    from tilespgemm_gb300 import _abi
    from tilespgemm_gb300 import matrices as M
    L = _abi.lib()
    for n in (100, 2049, 20000, 300000):
        st = L.tsg_check_bounded_wait(fresh.handle, n, 2000)
        assert st == _abi.ERR_DEVICE_TIMEOUT, (n, st)
        assert b"gave up" in L.tsg_last_error()
        _exact(fresh, M.laplacian_2d(48), "AA")


def _sweep(kind, call, after):
    """Arm the k-th allocation of `kind` to fail for k = 1, 2, ... until a call
    makes fewer allocations than k.  An armed failure either surfaces as
    TSG_ERR_OOM or hits an optional buffer the call can do without (step 1
    keeps wide tile-rows' bitmaps only when there is room), in which case the
    call must still succeed with the exact result (`call` checks it); after
    each one `after()` (an exact product on the same context) must pass.
    Returns the number of failures reported."""
    from tilespgemm_gb300 import TSGError, _abi
    L = _abi.lib()
    fails = 0
    for k in range(1, 400):
        assert L.tsg_inject_alloc_failure(kind, k) == _abi.OK
        try:
            call()
            fired = False
        except TSGError as e:
            assert e.status == _abi.ERR_OOM, (k, e)
            fired = True
        pending = L.tsg_alloc_failure_pending(kind)
        L.tsg_inject_alloc_failure(kind, 0)
        if not fired and pending > 0:
            return fails          # the call made fewer than k allocations
        fails += int(fired)
        after()
    raise AssertionError("the call made more than 400 allocations")


@pytest.mark.parametrize("op,out", [("AA", "host"), ("AAT", "device"), ("AA", "device")])
def test_every_pool_allocation_failure_is_reported(fresh, op, out):
    from tilespgemm_gb300 import matrices as M
    A = M.random_sparse(900, 900, 9, seed=31, empty_rows=0.1) if op == "AA" else M.rmat(10, 12, seed=9)

    def call():
        from tilespgemm_gb300.api import CSR
        oc, _ = fresh.spgemm_raw(A, op=op, out=out)
        try:
            C = oc.download()
        finally:
            oc.free()
        B = A
        if op == "AAT":
            tp, tr, tv = O.transpose(A)
            B = CSR(A.n, A.m, tp, tr, tv)
        rp, col, val = O.spgemm(A, B)
        assert np.array_equal(np.asarray(C.rowptr, np.int64), rp) and np.array_equal(C.col, col)
        assert np.array_equal(C.val, val)

    n = _sweep(0, call, lambda: _exact(fresh, A, op))
    assert n >= 10   # the call allocates at every stage: staging, tiles, step 1, step 2, numeric, output
    _exact(fresh, A, op)


def test_pinned_allocation_failure_is_reported(fresh):
    from tilespgemm_gb300 import matrices as M
    A = M.stencil_27(12, seed=2)          # dense enough C tiles for the early column download
    n = _sweep(1, lambda: fresh.spgemm(A, op="AA"), lambda: _exact(fresh, A, "AA"))
    assert n >= 3                          # row pointers, columns, values
    B = M.random_sparse(500, 500, 3, seed=4)   # sparse C tiles: the copies after the numeric step
    assert _sweep(1, lambda: fresh.spgemm(B, op="AA"), lambda: _exact(fresh, B, "AA")) >= 3


def test_batched_and_plan_allocation_failures(fresh):
    from tilespgemm_gb300 import matrices as M
    As = [M.random_sparse(60 + 17 * i, 60 + 17 * i, 5, seed=40 + i) for i in range(6)]
    after = lambda: _exact(fresh, As[0], "AA")  # noqa: E731
    assert _sweep(0, lambda: fresh.spgemm_batched(As, op="AA"), after) >= 5
    assert _sweep(1, lambda: fresh.spgemm_batched(As, op="AA"), after) >= 2

    def plan_call():
        p = fresh.plan(As[1], op="AA")
        try:
            p.execute(np.asarray(As[1].val))
        finally:
            p.close()

    assert _sweep(0, plan_call, after) >= 5
