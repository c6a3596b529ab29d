"""The CPU oracle against golden vectors generated by the reference's own code
(tests/golden/make_golden.py): pins the restatement before it checks the GPU."""
import numpy as np
import pytest

from conftest import assert_values_close, golden_names, load_case
from oracle import oracle as O

CASES = golden_names()


def test_goldens_present():
    assert len(CASES) >= 10


@pytest.mark.parametrize("name", CASES)
def test_csr_product_matches_reference_cpu(name):
    d = load_case(name)
    rp, col, val, bnd = O.spgemm(d["A"], d["B"], with_bound=True)
    assert np.array_equal(rp, d["c_rowptr"])
    assert np.array_equal(col, d["c_col"])
    if d["exact"]:
        assert np.array_equal(val, d["c_val"])
    else:
        assert_values_close(val, d["c_val"], bnd)


@pytest.mark.parametrize("name", [n for n in CASES if "AAT" in n])
def test_transpose_matches_reference(name):
    d = load_case(name)
    tp, tr, tv = O.transpose(d["A"])
    assert np.array_equal(tp, d["b_rowptr"])
    assert np.array_equal(tr, d["b_col"])
    assert np.array_equal(tv, d["b_val"])


@pytest.mark.parametrize("name", CASES)
def test_tile_structure_matches_reference(name):
    d = load_case(name)
    t = O.tile_csr(d["A"])
    assert np.array_equal(t["blkrowptr"], d["a_blkrowptr"])
    assert np.array_equal(t["blkcolidx"], d["a_blkcolidx"])
    tb = O.tile_csr(d["B"])
    assert np.array_equal(tb["blkrowptr"], d["tile_blkrowptrB"])
    assert np.array_equal(tb["blkcolidx"], d["tile_blkcolidxB"])


@pytest.mark.parametrize("name", CASES)
def test_tile_steps_match_reference(name):
    d = load_case(name)
    t = O.tile_spgemm(d["A"], d["B"])
    assert np.array_equal(t["blkrowptr"], d["blkrowptrC"])
    assert np.array_equal(t["blkcolidx"], d["blkcolidxC"])
    assert np.array_equal(t["nnzb"], d["nnzbC"])
    assert np.array_equal(t["ptr"], d["ptrC"])
    assert np.array_equal(t["col"], d["colC"])
    if d["exact"]:
        assert np.array_equal(t["val"], d["valC"])
    else:
        assert np.allclose(t["val"], d["valC"], rtol=1e-12, atol=1e-13)


@pytest.mark.parametrize("name", CASES)
def test_tiles_to_csr_gives_reference_csr(name):
    """The tile -> CSR output step, applied to the reference's own tile C,
    yields the reference CPU path's CSR C."""
    d = load_case(name)
    t = dict(blkrowptr=d["blkrowptrC"], blkcolidx=d["blkcolidxC"], nnzb=d["nnzbC"], ptr=d["ptrC"],
             col=d["colC"], val=d["valC"])
    rp, col, val = O.tiles_to_csr(int(d["m"]), t)
    assert np.array_equal(rp, d["c_rowptr"])
    assert np.array_equal(col, d["c_col"])
    if d["exact"]:
        assert np.array_equal(val, d["c_val"])


@pytest.mark.parametrize("name", CASES)
def test_thmkl_port_matches_reference(name):
    d = load_case(name)
    ic, jc, c = O.thmkl_rows(d["A"], d["B"], 0, int(d["m"]))
    assert np.array_equal(ic.astype(np.int64), d["c_rowptr"])
    assert np.array_equal(jc, d["c_col"])
    assert np.array_equal(c, d["c_val"]) or np.allclose(c, d["c_val"], rtol=1e-12, atol=1e-13)


def test_oracle_detects_planted_error():
    """A mistake planted in the oracle's output is caught by the golden comparison."""
    d = load_case("rand100_AA_refval")
    rp, col, val = O.spgemm(d["A"], d["B"])
    val = val.copy()
    val[7] += 1.0
    assert not np.array_equal(val, d["c_val"])


@pytest.mark.parametrize("name", ["rand100_AA", "rect77x130_AAT", "dup_unsorted64_AA", "emptyrows90_AA", "rmat8_AAT"])
def test_row_subset_oracle_matches_whole_product(name):
    """orc_spgemm_rows, the checker of sampled rows at full size, gives
    exactly the rows of the whole product (and of the reference's), for
    rows in any order with repeats."""
    d = load_case(name)
    rp, col, val, bnd = O.spgemm(d["A"], d["B"], with_bound=True)
    m = int(d["m"])
    rng = np.random.default_rng(3)
    rows = np.concatenate([rng.permutation(m)[: max(1, m // 3)], [0, m - 1, 0]])
    srp, scol, sval, sbnd = O.spgemm_rows(d["A"], d["B"], rows)
    assert srp[0] == 0 and srp.size == rows.size + 1
    for t, r in enumerate(rows):
        a, b = srp[t], srp[t + 1]
        assert np.array_equal(scol[a:b], col[rp[r]:rp[r + 1]])
        assert np.array_equal(sval[a:b].view(np.int64), val[rp[r]:rp[r + 1]].view(np.int64))
        assert np.array_equal(sbnd[a:b], bnd[rp[r]:rp[r + 1]])
        assert np.array_equal(scol[a:b], d["c_col"][d["c_rowptr"][r]:d["c_rowptr"][r + 1]])
