"""Numeric-only repeats through plans (tsg_plan_*): the same bits as a full
SpGEMM with the new values, for A*A, A*A^T and A*B, host and device values."""
import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu


def _newvals(A, seed):
    rng = np.random.default_rng(seed)
    return rng.uniform(-1.0, 1.0, A.nnz)


def _with(A, vals):
    from tilespgemm_gb300.api import CSR
    return CSR(A.m, A.n, A.rowptr, A.col, vals)


@pytest.mark.parametrize("op", ["AA", "AAT"])
def test_plan_matches_full_call(ctx, op):
    from tilespgemm_gb300 import matrices as M
    A = M.random_sparse(1500, 1500, 9, seed=31) if op == "AA" else M.random_sparse(900, 1300, 8, seed=32)
    plan = ctx.plan(A, op=op)
    assert plan.nnz > 0 and plan.device_bytes > 0
    for seed in range(3):
        v = _newvals(A, seed)
        Av = _with(A, v)
        C1 = plan.execute(v)
        C2 = ctx.spgemm(Av, op=op)
        assert np.array_equal(C1.rowptr, C2.rowptr) and np.array_equal(C1.col, C2.col)
        assert np.array_equal(C1.val, C2.val)
        B = Av if op == "AA" else _with(A, v)  # structure of B built by the oracle below
        if op == "AAT":
            from tilespgemm_gb300.api import CSR
            tp, tr, tv = O.transpose(Av)
            B = CSR(A.n, A.m, tp, tr, tv)
        rp, col, val = O.spgemm(Av, B)
        assert np.array_equal(C1.val, val)
    plan.close()


@pytest.mark.parametrize("op", ["AA", "AAT"])
def test_plan_host_output_dense_tiles(ctx, op):
    """C tiles of 8+ entries: a plan's host output writes C's column indices
    before the numeric step and copies them down beside it; the same bits
    as the full call and the oracle."""
    from tilespgemm_gb300 import matrices as M
    A = M.laplacian_2d(64) if op == "AA" else M.stencil_27(9, seed=4)
    plan = ctx.plan(A, op=op)
    for seed in range(2):
        v = _newvals(A, 40 + seed)
        Av = _with(A, v)
        C1 = plan.execute(v)
        C2 = ctx.spgemm(Av, op=op)
        assert np.array_equal(C1.rowptr, C2.rowptr) and np.array_equal(C1.col, C2.col)
        assert np.array_equal(C1.val, C2.val)
        tp, tr, tv = O.transpose(Av)
        from tilespgemm_gb300.api import CSR
        B = Av if op == "AA" else CSR(A.n, A.m, tp, tr, tv)
        rp, col, val = O.spgemm(Av, B)
        assert np.array_equal(np.asarray(C1.rowptr, np.int64), rp) and np.array_equal(C1.col, col)
        assert np.array_equal(C1.val, val)
    plan.close()


def test_plan_ab_and_device_values(ctx):
    import torch
    from tilespgemm_gb300 import matrices as M
    A = M.random_sparse(600, 800, 7, seed=33)
    B = M.random_sparse(800, 500, 6, seed=34)
    plan = ctx.plan(A, B, op="AB")
    va, vb = _newvals(A, 5), _newvals(B, 6)
    C1 = plan.execute(va, vb)
    oc, _ = plan.execute_raw(torch.from_numpy(va).cuda(), torch.from_numpy(vb).cuda(), out="device")
    C2 = oc.download()
    oc.free()
    rp, col, val = O.spgemm(_with(A, va), _with(B, vb))
    for C in (C1, C2):
        assert np.array_equal(np.asarray(C.rowptr, np.int64), rp) and np.array_equal(C.col, col)
        assert np.array_equal(C.val, val)
    plan.close()


def test_plan_outlives_device_operands(ctx):
    """A plan built from device tensors copies them: freeing them is safe."""
    import torch
    from tilespgemm_gb300 import matrices as M
    A = M.stencil_27(10, seed=2)
    Ad = A.to_device(0)
    plan = ctx.plan(Ad, op="AA")
    del Ad
    torch.cuda.empty_cache()
    v = _newvals(A, 9)
    C = plan.execute(v)
    rp, col, val = O.spgemm(_with(A, v), _with(A, v))
    assert np.array_equal(C.col, col) and np.array_equal(C.val, val)
    plan.close()


@pytest.mark.parametrize("op", ["AA", "AAT", "AB"])
def test_batched_plan_replay(ctx, op):
    """Batched plan: new values, graph replays (before and after tuning)
    give each instance the bits of its own full product."""
    from tilespgemm_gb300 import matrices as M
    sizes = [(40, 40), (300, 300), (17, 17), (1200, 1200), (64, 64)]
    if op == "AA":
        As = [M.random_sparse(m, m, 6, seed=60 + i) for i, (m, _) in enumerate(sizes)]
        Bs = None
    elif op == "AAT":
        As = [M.random_sparse(m, m + 37, 5, seed=70 + i) for i, (m, _) in enumerate(sizes)]
        Bs = None
    else:
        As = [M.random_sparse(m, m + 11, 5, seed=80 + i) for i, (m, _) in enumerate(sizes)]
        Bs = [M.random_sparse(m + 11, 200 + 13 * i, 4, seed=90 + i) for i, (m, _) in enumerate(sizes)]
    plan = ctx.plan_batched(As, Bs, op=op)
    assert plan.count == len(As)
    ao, bo = plan.value_offsets()
    assert ao[-1] == sum(A.nnz for A in As)
    for rnd in range(3):
        va = np.concatenate([_newvals(A, 100 * rnd + i) for i, A in enumerate(As)])
        vb = np.concatenate([_newvals(B, 200 * rnd + i) for i, B in enumerate(Bs)]) if Bs else None
        plan.set_values(va, vb)
        if rnd == 1:
            before = plan.settings()
            assert before["dense_tile_min"] == 160 and before["smem_acc_max"] == 24576
            assert plan.tune() > 0.0
            st = plan.settings()   # the tuner's pick: any of its candidates, same bits
            assert st["threads"] in (128, 256, 512) and st["walk"] in (1, 2, 3)
            assert (st["dense_tile_min"], st["smem_acc_max"], st["row_acc_max"]) in {
                (160, 24576, 65535), (96, 24576, 65535), (257, 24576, 65535), (160, 12288, 65535),
                (160, 65535, 65535), (160, 24576, 16384)}
        plan.replay()
        plan.replay()   # idempotent on the same values
        for i, A in enumerate(As):
            Ai = _with(A, va[ao[i]:ao[i + 1]])
            Bi = _with(Bs[i], vb[bo[i]:bo[i + 1]]) if Bs else None
            ref = ctx.spgemm(Ai, Bi, op=op)
            got = plan.result(i)
            assert np.array_equal(got.rowptr, np.asarray(ref.rowptr, np.int64))
            assert np.array_equal(got.col, ref.col)
            assert np.array_equal(got.val, ref.val)
    plan.close()


def test_plain_plan_replay(ctx):
    from tilespgemm_gb300 import matrices as M
    A = M.random_sparse(2500, 2500, 11, seed=99)
    plan = ctx.plan(A, op="AA")
    v = _newvals(A, 5)
    plan.set_values(v)
    plan.replay()
    ref = ctx.spgemm(_with(A, v), op="AA")
    got = plan.result(0)
    assert np.array_equal(got.col, ref.col) and np.array_equal(got.val, ref.val)
    plan.close()


def test_plan_replay_of_wide_rows_in_parts(built_lib):
    """Every row forced to the wide class (smem_acc_max=0, row_acc_max=0) in
    a C 20,000 columns wide: the parts path -- cut table, part walk -- runs
    inside the plan's captured graph (its table sized by the bound there)."""
    from tilespgemm_gb300 import Context
    from tilespgemm_gb300 import matrices as M
    A = M.random_sparse(600, 2000, 40, seed=51)
    B = M.random_sparse(2000, 20000, 20, seed=52)
    with Context(0, smem_acc_max=0, row_acc_max=0) as c:
        plan = c.plan(A, B, op="AB")
        for rnd in range(2):
            va, vb = _newvals(A, 10 + rnd), _newvals(B, 20 + rnd)
            plan.set_values(va, vb)
            plan.replay()
            got = plan.result(0)
            ref = c.spgemm(_with(A, va), _with(B, vb), op="AB")
            assert np.array_equal(got.col, ref.col) and np.array_equal(got.val, ref.val)
            rp, col, val = O.spgemm(_with(A, va), _with(B, vb))
            assert np.array_equal(got.col, col) and np.array_equal(got.val, val)
        plan.close()
