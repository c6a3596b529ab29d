"""The drop-in front ends of the C ABI, compiled as C:

* `tsg` (tilespgemm_gb300/cli/tsg.c), the reference driver's command line
  (`-d <dev> <A.mtx>`, main_spgemm-col.cu:4821-4853) with its
  results_tile.csv line (:5554-5559);
* the C binding INTEGRATION.md shows a maintainer adding to the reference's
  main, extracted from the document, wrapped in a main() that supplies the
  reference's variables, compiled with gcc -std=c99 against
  include/tilespgemm.h and linked to libtilespgemm.so.

Without a GPU they compile, link and refuse what the reference refuses;
with one (-m gpu) their outputs are checked against the oracle."""
import re
import shutil
import subprocess

import numpy as np
import pytest

from conftest import GOLDEN, ROOT

SNIPPET_MAIN = r"""
#include <stdio.h>
#include <stdint.h>
#include <string.h>
#include "tilespgemm.h"

#ifndef AAT
#define AAT 0
#endif

/* the reference's CSR struct (main_spgemm-col.cu:34-39) */
typedef struct { double *value; int *columnindex; int *rowpointer; } SMatrix;

int main(int argc, char **argv)
{
    int device_id = 0, rowA, colA, nnzA;
    SMatrix matrixA;
    tsg_csr L;
    memset(&L, 0, sizeof(L));
    if (argc < 2 || tsg_load_mtx(argv[1], &L, NULL) != TSG_OK) { fprintf(stderr, "load failed\n"); return 2; }
    rowA = L.m; colA = L.n; nnzA = (int)L.nnz;
    matrixA.rowpointer = (int *)L.row_ptr; matrixA.columnindex = L.col; matrixA.value = L.val;
    {
%s
    }
    tsg_csr_free(NULL, &L);
    return 0;
}
"""


def integration_snippet() -> str:
    text = (ROOT / "INTEGRATION.md").read_text()
    blocks = re.findall(r"```c\n(.*?)```", text, flags=re.S)
    assert blocks, "INTEGRATION.md has no C block"
    return "\n".join(line for line in blocks[0].splitlines() if not line.startswith("#include"))


@pytest.fixture(scope="module")
def snippet_bin(built_lib, tmp_path_factory):
    from tilespgemm_gb300 import build
    cc = shutil.which("gcc")
    if cc is None:
        pytest.skip("gcc not found")
    d = tmp_path_factory.mktemp("snippet")
    src = d / "snippet.c"
    src.write_text(SNIPPET_MAIN % integration_snippet())
    exe = d / "snippet"
    res = subprocess.run([cc, "-std=c99", "-Wall", "-Werror", f"-I{ROOT / 'include'}", str(src),
                          f"-L{build.LIBDIR}", "-ltilespgemm", f"-Wl,-rpath,{build.LIBDIR}", "-o", str(exe)],
                         capture_output=True, text=True)
    assert res.returncode == 0, res.stderr
    return exe


@pytest.fixture(scope="module")
def cli(built_lib):
    from tilespgemm_gb300 import build
    return build.build_cli()


def test_integration_snippet_compiles_and_links(snippet_bin):
    assert snippet_bin.exists()


README_MAIN = r"""
#include <stdint.h>
#include "tilespgemm.h"

int main(void)
{
    int32_t rowptr[3] = {0, 1, 2}, col[2] = {0, 1};
    double val[2] = {1.0, 2.0};
    int32_t m = 2, n = 2;
    int64_t nnz = 2;
    {
%s
    }
    return 0;
}
"""


def test_readme_c_example_compiles_and_links(built_lib, tmp_path):
    """The C example of README.md, given a 2 x 2 CSR, compiles with gcc
    -std=c99 -Wall -Werror against include/tilespgemm.h and links."""
    from tilespgemm_gb300 import build
    cc = shutil.which("gcc")
    if cc is None:
        pytest.skip("gcc not found")
    blocks = re.findall(r"```c\n(.*?)```", (ROOT / "README.md").read_text(), flags=re.S)
    assert blocks, "README.md has no C block"
    src = tmp_path / "readme.c"
    src.write_text(README_MAIN % blocks[0])
    res = subprocess.run([cc, "-std=c99", "-Wall", "-Werror", f"-I{ROOT / 'include'}", str(src),
                          f"-L{build.LIBDIR}", "-ltilespgemm", f"-Wl,-rpath,{build.LIBDIR}", "-o", str(tmp_path / "readme")],
                         capture_output=True, text=True)
    assert res.returncode == 0, res.stderr


def test_cli_usage_and_refusals(cli, tmp_path):
    res = subprocess.run([str(cli)], capture_output=True, text=True)
    assert res.returncode == 2 and "-d 0" in res.stderr
    # A*A on a non-square matrix and A*A^T on a symmetric one are refused, as
    # the reference refuses them, before any device work (exit 0, no line)
    rect = tmp_path / "rect.mtx"
    rect.write_text("%%MatrixMarket matrix coordinate real general\n2 3 2\n1 1 1.0\n2 3 2.0\n")
    res = subprocess.run([str(cli), "-d", "0", str(rect)], capture_output=True, text=True, cwd=tmp_path)
    assert res.returncode == 0 and "rowA == colA" in res.stdout
    sym = GOLDEN / "mtx" / "symmetric_real.mtx"
    res = subprocess.run([str(cli), "-d", "0", "--aat", str(sym)], capture_output=True, text=True, cwd=tmp_path)
    assert res.returncode == 0 and "symmetric" in res.stdout
    assert not (tmp_path / "results_tile.csv").exists()
    # a file that does not load: a library error, exit 1
    res = subprocess.run([str(cli), "-d", "0", str(tmp_path / "missing.mtx")], capture_output=True, text=True)
    assert res.returncode == 1


def _write_mtx(path, A):
    rows = np.repeat(np.arange(A.m), np.diff(np.asarray(A.rowptr)))
    with open(path, "w") as f:
        f.write("%%MatrixMarket matrix coordinate real general\n")
        f.write(f"{A.m} {A.n} {A.nnz}\n")
        for r, c, v in zip(rows, A.col, A.val):
            f.write(f"{r + 1} {c + 1} {float(v)!r}\n")


@pytest.mark.gpu
@pytest.mark.parametrize("aat", [False, True])
def test_cli_results_line(cli, tmp_path, aat):
    """The results_tile.csv line: nnzCub and nnzC of the reference's product
    (values i % 10, as the reference sets them), compression = nnzCub/nnzC."""
    from oracle import oracle as O
    from tilespgemm_gb300 import matrices as M
    from tilespgemm_gb300.api import CSR
    A = M.random_sparse(700, 500, 7, seed=21) if aat else M.laplacian_2d(40)
    path = tmp_path / "a.mtx"
    _write_mtx(path, A)
    args = [str(cli), "-d", "0", "--repeat", "3"] + (["--aat"] if aat else []) + [str(path)]
    res = subprocess.run(args, capture_output=True, text=True, cwd=tmp_path)
    assert res.returncode == 0, res.stdout + res.stderr
    line = (tmp_path / "results_tile.csv").read_text().strip().splitlines()[-1].split(",")
    assert line[0] == str(path) and int(line[1]) == A.m and int(line[2]) == A.n and int(line[3]) == A.nnz
    B = A
    if aat:
        tp, tr, tv = O.transpose(A)
        B = CSR(A.n, A.m, tp, tr, tv)
    rp, _, _ = O.spgemm(A, B)
    cub = O.nnzcub(A, B)
    assert int(line[4]) == cub and int(line[5]) == int(rp[-1])
    assert abs(float(line[6]) - cub / rp[-1]) < 1e-5
    assert float(line[7]) > 0 and float(line[8]) > 0


@pytest.mark.gpu
def test_integration_snippet_runs(snippet_bin, tmp_path):
    from oracle import oracle as O
    from tilespgemm_gb300 import matrices as M
    A = M.stencil_27(9, seed=4)
    path = tmp_path / "s.mtx"
    _write_mtx(path, A)
    res = subprocess.run([str(snippet_bin), str(path)], capture_output=True, text=True)
    assert res.returncode == 0, res.stdout + res.stderr
    rp, _, _ = O.spgemm(A, A)
    assert f"nnzC = {int(rp[-1])}," in res.stdout
