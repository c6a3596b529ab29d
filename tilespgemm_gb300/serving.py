"""Serving (tsg_server_*): continuous batching of SpGEMM requests on one GPU,
and the Poisson request stream it is measured on.

    with Server(workers=4, budget_gb=64) as srv:
        rid = srv.submit(A, op="AA", key=pattern_hash)   # key: reuse the symbolic result
        C, info = srv.wait(rid)

The stream: Poisson arrivals (mean 2,000 requests/s), half 2D 5-point
Laplacians (grid side uniform in 32..512) and half R-MAT matrices (2^12..2^18
rows, 8..32 nnz/row), half A*A and half A*A^T, 30% of requests repeating an
earlier pattern with new values (numeric-only), admitted under a 64 GB
device-memory budget.
"""
from __future__ import annotations

import ctypes as C
import threading
import time

import numpy as np

from . import _abi
from ._abi import TSGError, check, lib
from .api import CSR, _download

_OPS = {"AB": _abi.OP_AB, "AA": _abi.OP_AA, "AAT": _abi.OP_AAT}


class Server:
    def __init__(self, device: int = 0, workers: int = 4, max_batch: int = 32, budget_gb: float = 64.0,
                 plan_cache_gb: float = 8.0):
        o = _abi.tsg_server_opts()
        lib().tsg_server_opts_default(C.byref(o))
        o.device, o.workers, o.max_batch = device, workers, max_batch
        o.budget_bytes = int(budget_gb * (1 << 30))
        o.plan_cache_bytes = int(plan_cache_gb * (1 << 30))
        h = C.c_void_p()
        check(lib().tsg_server_create(C.byref(o), C.byref(h)))
        self.handle = h
        self._keep: dict[int, list] = {}
        self._lock = threading.Lock()

    def submit(self, A: CSR, op: str = "AA", B: CSR | None = None, key: int = 0) -> int:
        a, ka = A._tsg()
        b_ptr, kb = None, []
        if B is not None:
            b, kb = B._tsg()
            b_ptr = C.byref(b)
        rid = C.c_int64()
        check(lib().tsg_server_submit(self.handle, _OPS[op], C.byref(a), b_ptr, C.c_uint64(key), C.byref(rid)))
        with self._lock:
            self._keep[rid.value] = [ka, kb]       # operands must outlive the request
        return rid.value

    def wait(self, rid: int, download: bool = True) -> tuple[CSR | None, dict]:
        """Result of request `rid` (a host CSR; None with download=False,
        which only releases it) and its timing record."""
        c = _abi.tsg_csr()
        info = _abi.tsg_server_result()
        st = lib().tsg_server_wait(self.handle, C.c_int64(rid), C.byref(c), C.byref(info))
        if st != _abi.ERR_INVALID_ARG:   # returned (invalid: unknown, or another thread waits for it)
            with self._lock:
                self._keep.pop(rid, None)
        check(st)
        d = info.as_dict()
        d["nnz"] = int(c.nnz)
        res = _download(None, c) if download else None
        lib().tsg_csr_free(None, C.byref(c))
        return res, d

    def wait_any(self, download: bool = True) -> tuple[int, CSR | None, dict]:
        """The next request to complete (completion order): its id, result
        (None with download=False) and timing record."""
        c = _abi.tsg_csr()
        info = _abi.tsg_server_result()
        rid = C.c_int64()
        st = lib().tsg_server_wait_any(self.handle, C.byref(rid), C.byref(c), C.byref(info))
        check(st)
        with self._lock:
            self._keep.pop(rid.value, None)
        d = info.as_dict()
        d["nnz"] = int(c.nnz)
        res = _download(None, c) if download else None
        lib().tsg_csr_free(None, C.byref(c))
        return rid.value, res, d

    def close(self) -> None:
        if self.handle:
            lib().tsg_server_destroy(self.handle)
            self.handle = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()


def _build_request(spec: dict) -> CSR:
    """Matrix of one stream request from its drawn spec (runs in a worker process)."""
    from . import matrices as M
    vr = np.random.Generator(np.random.Philox(spec["vseed"]))
    if spec["kind"].startswith("lap"):
        A = M.laplacian_2d(spec["side"])
    else:
        A = M.rmat(spec["scale"], spec["ef"], seed=spec["mseed"])
    return CSR(A.m, A.n, A.rowptr, A.col, vr.uniform(-1.0, 1.0, A.nnz))


def make_stream(n_requests: int, seed: int = 1, rate: float = 2000.0, repeat_frac: float = 0.3,
                lap_side=(32, 512), rmat_scale=(12, 18), rmat_edge=(8, 32), procs: int = 0, key_base: int = 0):
    """The seeded request stream: list of dicts (t, A, op, key, kind).

    Arrival gaps are exponential (Poisson arrivals at `rate`/s).  With
    probability `repeat_frac` a request repeats an earlier request's pattern
    (same key) with new values; otherwise it is a fresh 2D Laplacian or R-MAT
    operand, A*A or A*A^T with equal odds.  All draws are made first, in one
    sequential pass; the operands are then built, in `procs` spawned worker
    processes when procs > 1 (start those before the first GPU call).
    Pattern keys are key_base + 1, key_base + 2, ... (streams sent to one
    server must not share keys)."""
    rng = np.random.Generator(np.random.Philox(seed))
    t = 0.0
    specs = []
    for i in range(n_requests):
        t += rng.exponential(1.0 / rate)
        vseed = int(rng.integers(1, 2 ** 62))
        if specs and rng.random() < repeat_frac:
            base = specs[int(rng.integers(0, len(specs)))]
            specs.append(dict(base, t=t, vseed=vseed, kind=base["kind"].replace("-repeat", "") + "-repeat"))
            continue
        op = "AA" if rng.random() < 0.5 else "AAT"
        if rng.random() < 0.5:
            side = int(rng.integers(lap_side[0], lap_side[1] + 1))
            specs.append(dict(t=t, vseed=vseed, op=op, key=key_base + i + 1, kind=f"lap{side}", side=side))
        else:
            scale = int(rng.integers(rmat_scale[0], rmat_scale[1] + 1))
            ef = int(rng.integers(rmat_edge[0], rmat_edge[1] + 1))
            specs.append(dict(t=t, vseed=vseed, op=op, key=key_base + i + 1, kind=f"rmat{scale}x{ef}", scale=scale, ef=ef,
                              mseed=int(rng.integers(1, 2 ** 31))))
    if procs > 1 and len(specs) > 1:
        import multiprocessing as mp
        with mp.get_context("spawn").Pool(procs) as pool:
            mats = pool.map(_build_request, specs, chunksize=1)
    else:
        mats = [_build_request(sp) for sp in specs]
    return [dict(t=sp["t"], A=A, op=sp["op"], key=sp["key"], kind=sp["kind"]) for sp, A in zip(specs, mats)]


def run_stream(srv: Server, reqs: list, realtime: bool = True, download: bool = True) -> dict:
    """Submit the stream at its arrival times; collect results and latencies.

    A request the budget refuses at submission (TSG_ERR_BUDGET) is counted
    in `refused` and has no latency; other errors propagate."""
    ids = [None] * len(reqs)
    results = [None] * len(reqs)
    errors: list = []
    where: dict[int, int] = {}       # request id -> stream index, filled by the submitter
    state = {"submitted": 0, "done": False}
    t0 = time.perf_counter()

    def collector():
        # results are taken in completion order and released at once, so
        # host memory holds only the requests in flight
        try:
            got = 0
            while True:
                if got < state["submitted"]:
                    rid, res, d = srv.wait_any(download=download)
                    while rid not in where:          # its submit call is still returning
                        time.sleep(0.0001)
                    results[where[rid]] = (res, d)
                    got += 1
                elif state["done"]:
                    break
                else:
                    time.sleep(0.0002)
        except BaseException as e:   # surfaced after join
            errors.append(e)

    th = threading.Thread(target=collector)
    th.start()
    try:
        for i, r in enumerate(reqs):
            if realtime:
                dt = r["t"] - (time.perf_counter() - t0)
                if dt > 0:
                    time.sleep(dt)
            try:
                rid = srv.submit(r["A"], op=r["op"], key=r["key"])
                ids[i] = rid
                where[rid] = i
                state["submitted"] += 1
            except TSGError as e:
                if e.status != _abi.ERR_BUDGET:
                    raise
                ids[i] = -1
    finally:
        for i in range(len(ids)):
            if ids[i] is None:
                ids[i] = -1
        state["done"] = True
        th.join()
    if errors:
        raise errors[0]
    wall = time.perf_counter() - t0
    done = [res for res in results if res is not None]
    lat = np.array([res[1]["latency_ms"] for res in done]) if done else np.zeros(1)
    return dict(n=len(reqs), completed=len(done), refused=sum(1 for x in ids if x < 0), wall_s=wall,
                throughput_rps=len(done) / wall, p50_ms=float(np.percentile(lat, 50)),
                p99_ms=float(np.percentile(lat, 99)), mean_ms=float(lat.mean()),
                numeric_only=int(sum(res[1]["numeric_only"] for res in done)), results=results)
