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
from ._abi import check, lib
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

    def wait(self, rid: int) -> tuple[CSR, dict]:
        c = _abi.tsg_csr()
        info = _abi.tsg_server_result()
        st = lib().tsg_server_wait(self.handle, C.c_int64(rid), C.byref(c), C.byref(info))
        with self._lock:
            self._keep.pop(rid, None)
        check(st)
        res = _download(None, c)
        lib().tsg_csr_free(None, C.byref(c))
        return res, info.as_dict()

    def close(self) -> None:
        if self.handle:
            lib().tsg_server_destroy(self.handle)
            self.handle = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()


def make_stream(n_requests: int, seed: int = 1, rate: float = 2000.0, repeat_frac: float = 0.3,
                lap_side=(32, 512), rmat_scale=(12, 18), rmat_edge=(8, 32)):
    """The seeded request stream: list of dicts (t_arrival, A, op, key, kind)."""
    from . import matrices as M
    rng = np.random.Generator(np.random.Philox(seed))
    t = 0.0
    reqs = []
    for i in range(n_requests):
        t += rng.exponential(1.0 / rate)
        if reqs and rng.random() < repeat_frac:
            base = reqs[int(rng.integers(0, len(reqs)))]
            A0 = base["A"]
            A = CSR(A0.m, A0.n, A0.rowptr, A0.col, rng.uniform(-1.0, 1.0, A0.nnz))
            reqs.append(dict(t=t, A=A, op=base["op"], key=base["key"], kind=base["kind"] + "-repeat"))
            continue
        op = "AA" if rng.random() < 0.5 else "AAT"
        if rng.random() < 0.5:
            side = int(rng.integers(lap_side[0], lap_side[1] + 1))
            A = M.laplacian_2d(side)
            A = CSR(A.m, A.n, A.rowptr, A.col, rng.uniform(-1.0, 1.0, A.nnz))
            kind = f"lap{side}"
        else:
            scale = int(rng.integers(rmat_scale[0], rmat_scale[1] + 1))
            ef = int(rng.integers(rmat_edge[0], rmat_edge[1] + 1))
            A = M.rmat(scale, ef, seed=int(rng.integers(1, 2 ** 31)))
            kind = f"rmat{scale}x{ef}"
        reqs.append(dict(t=t, A=A, op=op, key=i + 1, kind=kind))
    return reqs


def run_stream(srv: Server, reqs: list, realtime: bool = True) -> dict:
    """Submit the stream at its arrival times; collect results and latencies."""
    ids = [None] * len(reqs)
    results = [None] * len(reqs)
    t0 = time.perf_counter()

    def collector():
        for i in range(len(reqs)):
            while ids[i] is None:
                time.sleep(0.0001)
            C_, info = srv.wait(ids[i])
            results[i] = (C_, info)

    th = threading.Thread(target=collector)
    th.start()
    for i, r in enumerate(reqs):
        if realtime:
            dt = r["t"] - (time.perf_counter() - t0)
            if dt > 0:
                time.sleep(dt)
        ids[i] = srv.submit(r["A"], op=r["op"], key=r["key"])
    th.join()
    wall = time.perf_counter() - t0
    lat = np.array([res[1]["latency_ms"] for res in results])
    flops = 0.0
    return dict(n=len(reqs), wall_s=wall, throughput_rps=len(reqs) / wall, p50_ms=float(np.percentile(lat, 50)),
                p99_ms=float(np.percentile(lat, 99)), mean_ms=float(lat.mean()),
                numeric_only=int(sum(res[1]["numeric_only"] for res in results)), flops=flops, results=results)
