"""Shared fixtures.  Tests marked `gpu` need a GB300; everything else runs on CPU."""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]
GOLDEN = ROOT / "tests" / "golden"
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a GB300 GPU (sm_103a)")


def golden_names() -> list[str]:
    return sorted(p.stem for p in GOLDEN.glob("*.npz") if not p.stem.startswith("mtx_"))


def load_case(name: str) -> dict:
    from tilespgemm_gb300.api import CSR
    d = dict(np.load(GOLDEN / f"{name}.npz"))
    d["op"] = str(d["op"])
    m, n = int(d["m"]), int(d["n"])
    d["A"] = CSR(m, n, d["a_rowptr"].astype(np.int64), d["a_col"].astype(np.int32), d["a_val"])
    bm = n if d["op"] == "AA" or d["op"] == "AAT" else None
    d["B"] = CSR(int(d["b_rowptr"].size - 1), (m if d["op"] == "AAT" else n), d["b_rowptr"].astype(np.int64),
                 d["b_col"].astype(np.int32), d["b_val"])
    del bm
    d["exact"] = name.endswith("_refval")
    return d


def assert_values_close(got: np.ndarray, ref: np.ndarray, bound: np.ndarray, rtol: float = 1e-12) -> None:
    """Per-entry |got - ref| <= rtol * sum|a||b| (the stated tolerance: 1e-12
    relative to the magnitude of the products that make the entry, which stays
    well-posed when values cancel)."""
    err = np.abs(got - ref)
    lim = rtol * np.maximum(bound, np.abs(ref))
    bad = np.nonzero(err > lim)[0]
    assert bad.size == 0, f"{bad.size} entries out of tolerance, first at {bad[:5]}: {got[bad[:5]]} vs {ref[bad[:5]]}"


@pytest.fixture(scope="session")
def built_lib():
    """libtilespgemm.so, built here if missing (nvcc cross-compiles without a GPU)."""
    from tilespgemm_gb300 import build
    if not build.LIB.exists():
        build.build_library()
    return build.LIB


@pytest.fixture(scope="session")
def ctx(built_lib):
    """A context on the tiled pipeline (the small-product path off, so that
    small test matrices exercise the tiled kernels; tests/test_small_gpu.py
    covers that path)."""
    from tilespgemm_gb300 import Context
    c = Context(0, small_path=0)
    yield c
    c.close()
