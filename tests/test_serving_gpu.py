"""Serving: results are the same alone and in the mix (bit for bit), repeats
with a known pattern run numeric-only, and the budget refuses what cannot fit."""
import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu


def _req_set():
    from tilespgemm_gb300 import matrices as M
    from tilespgemm_gb300.api import CSR
    rng = np.random.default_rng(5)
    out = []
    for i in range(24):
        if i % 3 == 0:
            A = M.laplacian_2d(int(rng.integers(8, 40)))
        elif i % 3 == 1:
            A = M.rmat(int(rng.integers(6, 10)), 8, seed=i + 1)
        else:
            A = M.random_sparse(int(rng.integers(20, 300)), int(rng.integers(20, 300)), 5, seed=i)
        A = CSR(A.m, A.n, A.rowptr, A.col, rng.uniform(-1, 1, A.nnz))
        op = "AAT" if (i % 2 or A.m != A.n) else "AA"
        out.append((A, op, (i + 1) if i % 4 == 0 else 0))
    return out


def test_same_alone_and_in_the_mix(built_lib):
    from tilespgemm_gb300.serving import Server
    reqs = _req_set()
    with Server(workers=3, max_batch=8, budget_gb=4) as srv:
        alone = []
        for A, op, key in reqs:
            alone.append(srv.wait(srv.submit(A, op=op, key=key))[0])
        ids = [srv.submit(A, op=op, key=key) for A, op, key in reqs]     # all at once
        mixed = [srv.wait(i) for i in ids]
    batched = sum(1 for _, info in mixed if info["batched_with"] > 1)
    assert batched > 0, "keyless requests taken together should share a batched product"
    for (A, op, _), Ca, (Cm, info) in zip(reqs, alone, mixed):
        assert np.array_equal(Ca.rowptr, Cm.rowptr) and np.array_equal(Ca.col, Cm.col)
        assert np.array_equal(Ca.val, Cm.val)
        from tilespgemm_gb300.api import CSR
        B = A if op == "AA" else CSR(A.n, A.m, *O.transpose(A))
        rp, col, val = O.spgemm(A, B)
        assert np.array_equal(Cm.col, col) and np.array_equal(Cm.val, val)


def test_repeats_run_numeric_only(built_lib):
    from tilespgemm_gb300 import matrices as M
    from tilespgemm_gb300.api import CSR
    from tilespgemm_gb300.serving import Server
    A = M.rmat(9, 8, seed=4)
    rng = np.random.default_rng(1)
    with Server(workers=2) as srv:
        _, i1 = srv.wait(srv.submit(A, op="AAT", key=77))
        A2 = CSR(A.m, A.n, A.rowptr, A.col, rng.uniform(-1, 1, A.nnz))
        C2, i2 = srv.wait(srv.submit(A2, op="AAT", key=77))
    assert i1["numeric_only"] == 0 and i2["numeric_only"] == 1
    B2 = CSR(A2.n, A2.m, *O.transpose(A2))
    rp, col, val = O.spgemm(A2, B2)
    assert np.array_equal(C2.col, col) and np.array_equal(C2.val, val)


def test_key_reused_for_another_pattern(built_lib):
    """A key whose pattern changes rebuilds its plan (fingerprint check)."""
    from tilespgemm_gb300 import matrices as M
    from tilespgemm_gb300.serving import Server
    A1 = M.rmat(9, 8, seed=4)
    A2 = M.rmat(9, 8, seed=5)
    with Server(workers=1) as srv:
        srv.wait(srv.submit(A1, op="AA", key=5))
        C2, info = srv.wait(srv.submit(A2, op="AA", key=5))
    assert info["numeric_only"] == 0
    rp, col, val = O.spgemm(A2, A2)
    assert np.array_equal(C2.col, col) and np.array_equal(C2.val, val)


def test_budget_refuses_oversized(built_lib):
    from tilespgemm_gb300 import TSGError
    from tilespgemm_gb300 import matrices as M
    from tilespgemm_gb300.serving import Server
    A = M.laplacian_2d(200)
    with Server(workers=1, budget_gb=0.001) as srv:
        with pytest.raises(TSGError) as e:
            srv.submit(A, op="AA")
        assert e.value.status == 10


def test_wait_any_returns_every_request_once(built_lib):
    """Completion-order collection gives each submitted request exactly once,
    with the same result as waiting for it by id; with nothing outstanding
    it reports an invalid argument."""
    from tilespgemm_gb300 import TSGError
    from tilespgemm_gb300.serving import Server
    reqs = _req_set()
    with Server(workers=3, max_batch=8, budget_gb=4) as srv:
        alone = [srv.wait(srv.submit(A, op=op, key=key))[0] for A, op, key in reqs]
        ids = [srv.submit(A, op=op, key=key) for A, op, key in reqs]
        got = {}
        for _ in ids:
            rid, C, info = srv.wait_any()
            assert rid not in got
            got[rid] = C
        with pytest.raises(TSGError) as e:
            srv.wait_any()
        assert e.value.status == 1
    assert sorted(got) == sorted(ids)
    for rid, Ca in zip(ids, alone):
        Cm = got[rid]
        assert np.array_equal(Ca.rowptr, Cm.rowptr) and np.array_equal(Ca.col, Cm.col)
        assert np.array_equal(Ca.val, Cm.val)


def test_run_stream_collects_in_completion_order(built_lib):
    from tilespgemm_gb300.serving import Server, make_stream, run_stream
    reqs = make_stream(12, seed=3, rate=500.0, lap_side=(16, 48), rmat_scale=(8, 10))
    with Server(workers=2, budget_gb=4) as srv:
        st = run_stream(srv, reqs, realtime=True, download=True)
    assert st["completed"] + st["refused"] == 12 and st["refused"] == 0
    for r, res in zip(reqs, st["results"]):
        C, info = res
        A = r["A"]
        from tilespgemm_gb300.api import CSR
        B = A if r["op"] == "AA" else CSR(A.n, A.m, *O.transpose(A))
        rp, col, val = O.spgemm(A, B)
        assert np.array_equal(C.col, col) and np.array_equal(C.val, val)
        assert info["latency_ms"] >= 0.0
