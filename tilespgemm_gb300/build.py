"""Build recipe for libtilespgemm.so (sm_103a) and the CPU oracle library.

The CUDA library is compiled in-tree with nvcc, one translation unit per
process in parallel, for exactly one target: ``-gencode
arch=compute_103a,code=sm_103a`` (GB300).  The CUDA runtime is linked
statically so the library loads without a toolkit on the library path.

The command-line front end (``cli/tsg.c``, plain C) is linked against it
as ``_lib/tsg``.

The oracle (``oracle/tsg_oracle.c``) is test infrastructure; it is built
beside it as ``oracle/liboracle.so`` so that tests and the CPU-baseline leg
of ``bench.py`` can load it.  When a reference checkout is present, the
reference's own CPU code is built into ``oracle/_ref`` by
``oracle/build_ref.sh``.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
OBJ = PKG / "_build"
LIBDIR = PKG / "_lib"
LIB = LIBDIR / "libtilespgemm.so"
ORACLE_SRC = ROOT / "oracle" / "tsg_oracle.c"
ORACLE_LIB = ROOT / "oracle" / "liboracle.so"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-Wall",
              "--expt-relaxed-constexpr", f"-I{ROOT / 'include'}", f"-I{CSRC}"]


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found: the CUDA 13 toolkit is required to build libtilespgemm.so")


def _run(cmd: list[str]) -> None:
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"command failed ({res.returncode}): {' '.join(cmd)}\n{res.stdout}\n{res.stderr}")


def _stale(out: Path, deps: list[Path]) -> bool:
    if not out.exists():
        return True
    t = out.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps)


def build_library(verbose: bool = False, jobs: int | None = None) -> Path:
    nvcc = _nvcc()
    OBJ.mkdir(exist_ok=True)
    LIBDIR.mkdir(exist_ok=True)
    sources = sorted(CSRC.glob("*.cu")) + sorted(CSRC.glob("*.cpp"))
    headers = sorted(CSRC.glob("*.cuh")) + sorted((ROOT / "include").glob("*.h"))
    jobs_to_run = []
    objs = []
    for src in sources:
        obj = OBJ / (src.name + ".o")
        objs.append(obj)
        if _stale(obj, [src] + headers):
            cmd = [nvcc, *ARCH, *NVCC_FLAGS, "-c", str(src), "-o", str(obj)]
            if src.suffix == ".cpp":
                cmd = [nvcc, *NVCC_FLAGS, "-x", "c++", "-c", str(src), "-o", str(obj)]
            jobs_to_run.append(cmd)
    if jobs_to_run:
        n = jobs or min(len(jobs_to_run), os.cpu_count() or 4)
        with cf.ThreadPoolExecutor(max_workers=n) as ex:
            for cmd, fut in [(c, ex.submit(_run, c)) for c in jobs_to_run]:
                fut.result()
                if verbose:
                    print(" ".join(cmd), file=sys.stderr)
    if jobs_to_run or _stale(LIB, objs):
        _run([nvcc, *ARCH, "-shared", "-cudart", "static", "-o", str(LIB), *map(str, objs)])
    return LIB


CLI_SRC = PKG / "cli" / "tsg.c"
CLI = LIBDIR / "tsg"


def build_cli() -> Path:
    """The command-line front end (plain C99 against include/tilespgemm.h),
    linked to libtilespgemm.so beside it."""
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        raise RuntimeError("gcc not found")
    if _stale(CLI, [CLI_SRC, LIB, ROOT / "include" / "tilespgemm.h"]):
        _run([cc, "-std=c99", "-D_POSIX_C_SOURCE=200809L", "-O2", "-Wall", "-Wextra", "-Werror",
              f"-I{ROOT / 'include'}", str(CLI_SRC), f"-L{LIBDIR}", "-ltilespgemm", "-Wl,-rpath,$ORIGIN",
              "-o", str(CLI)])
    return CLI


def build_oracle() -> Path:
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        raise RuntimeError("gcc not found")
    if _stale(ORACLE_LIB, [ORACLE_SRC]):
        _run([cc, "-O3", "-fopenmp", "-ffp-contract=off", "-fPIC", "-shared", "-Wall",
              str(ORACLE_SRC), "-o", str(ORACLE_LIB), "-lm"])
    return ORACLE_LIB


def build_reference() -> bool:
    """Build the reference's CPU code into oracle/_ref with the oracle's
    recipe (oracle/build_ref.sh), which knows where a reference checkout may
    sit and does nothing where there is none.  True when the libraries exist."""
    out = ROOT / "oracle" / "_ref"
    have = lambda: (out / "libthmkl_ref.so").exists() and (out / "libstir_ref.so").exists()  # noqa: E731
    recipe = [ROOT / "oracle" / "build_ref.sh", ROOT / "oracle" / "ref_shim_stir.cu"]
    if not have() or _stale(out / "libstir_ref.so", recipe) or _stale(out / "libthmkl_ref.so", recipe):
        _run(["bash", str(ROOT / "oracle" / "build_ref.sh")])
    return have()


def build_all(verbose: bool = False) -> None:
    build_library(verbose=verbose)
    build_cli()
    build_oracle()
    build_reference()


if __name__ == "__main__":
    build_all(verbose=True)
    print(LIB)
