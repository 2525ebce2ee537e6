"""The oracle (oracle/kdtree_oracle.c) against the reference's own outputs.

Fixtures in tests/golden/ were produced by running the reference's CPU
KD-tree (tests/golden/make_golden.py); here the C restatement must reproduce
them bit for bit -- layout, distances and indices, tie order included."""
import numpy as np
import pytest

from golden_util import inputs_of, rows
from make_golden import CASES, digest

NAMES = [c[0] for c in CASES]


@pytest.mark.parametrize("name", NAMES)
def test_oracle_matches_reference(name, oracle, golden):
    case = golden[name]
    ref, q = inputs_of(case)
    lay = oracle.build_tree(ref, int(case["levels"]))
    k = int(case["k"])
    d, i = oracle.query_tree(lay, q, k)
    r = rows(case)
    if str(case["kind"]) != "normal1e3":
        # Coordinates tie: the reference's std::sort orders tied points in an
        # unspecified way and the oracle by original index, so the trees (and
        # hence the visit order that breaks distance ties) differ.  The
        # distances must still agree bitwise, the indices up to ties.
        cmp = oracle.compare_knn(case["dists"], case["idx"], d[:r], i[:r])
        assert cmp.ok, cmp
        return
    np.testing.assert_array_equal(d[:r], case["dists"])
    np.testing.assert_array_equal(i[:r], case["idx"])
    assert digest(d, i) == str(case["output_sha"])
    if "perm" in case:
        # tie-free coordinates: the layout is unique and must be identical
        np.testing.assert_array_equal(lay.structured, case["structured"])
        np.testing.assert_array_equal(lay.perm, case["perm"])
        np.testing.assert_array_equal(lay.medians, case["medians"])
        np.testing.assert_array_equal(lay.axes, case["axes"])
        np.testing.assert_array_equal(lay.leaf_off[: len(case["leaf_off"])], case["leaf_off"])
        np.testing.assert_array_equal(lay.leaf_cnt[: len(case["leaf_cnt"])], case["leaf_cnt"])


@pytest.mark.parametrize("name", [n for n in NAMES if "config1" not in n])
def test_brute_force_agrees_with_reference_up_to_ties(name, oracle, golden):
    """The canonical answer (ties -> lower index) differs from the reference
    only inside groups of exactly equal distance."""
    case = golden[name]
    ref, q = inputs_of(case)
    bd, bi = oracle.brute(ref, q, int(case["k"]))
    cmp = oracle.compare_knn(case["dists"], case["idx"], bd, bi)
    assert cmp.ok, cmp
    if str(case["kind"]) != "normal1e3":
        assert cmp.tie_queries > 0  # the tie fixtures really exercise ties


def test_oracle_plants_a_mistake_and_catches_it(oracle, golden):
    """The comparison is not vacuous: a planted swap is reported."""
    case = golden["grid_f32_d3_n1000_q200_k10"]
    d = case["dists"].copy()
    i = case["idx"].copy()
    i[3, 2], i[3, 5] = i[3, 5], i[3, 2]
    cmp = oracle.compare_knn(case["dists"], case["idx"], d, i)
    assert cmp.mismatches > 0
    d[7, 0] = np.nextafter(d[7, 0], np.float32(np.inf))
    assert oracle.compare_knn(case["dists"], case["idx"], d, case["idx"]).dist_bit_mismatch == 1


def test_ran_out_of_points(oracle):
    pts = np.random.default_rng(1).standard_normal((10, 3)).astype(np.float32)
    with pytest.raises(RuntimeError):
        oracle.build_tree(pts, levels=6)


def test_fp64_helpers(oracle):
    rng = np.random.default_rng(2)
    ref = rng.standard_normal((500, 8)).astype(np.float32)
    q = rng.standard_normal((40, 8)).astype(np.float32)
    d64, i64 = oracle.brute_f64(ref, q, 5)
    bd, bi = oracle.brute(ref, q, 5)
    assert (i64 == bi).mean() > 0.99
    np.testing.assert_allclose(oracle.recompute_f64(ref, q, bi), bd, rtol=1e-5)


@pytest.mark.parametrize("case", [c for c in CASES if c[3] <= 10000], ids=lambda c: c[0])
def test_fixtures_regenerate_from_the_reference(case, oracle, golden):
    """Where the reference's own CPU code is built (oracle/_ref, compiled from
    its sources in the checkout), every fixture regenerates bit for bit:
    inputs, layout and query outputs."""
    if not oracle.ref_available():
        pytest.skip("reference sources are not built here")
    from make_golden import golden_inputs
    name, dtype, d, n, nq, k, levels, kind, full = case
    ref, q = golden_inputs(name, dtype, d, n, nq, kind)
    tree = oracle.RefTree(ref, levels)
    lay = tree.layout()
    dists, idx = tree.query(q, k)
    z = golden[name]
    assert str(z["input_sha"]) == digest(ref, q)
    assert str(z["layout_sha"]) == digest(lay.structured, lay.perm, lay.medians, lay.axes, lay.leaf_off, lay.leaf_cnt)
    assert str(z["output_sha"]) == digest(dists, idx)


@pytest.mark.parametrize("d", [1, 2, 3, 4, 5, 6, 7, 8])
@pytest.mark.parametrize("dtype", [np.float32, np.float64])
def test_restatement_equals_reference_on_fresh_clouds(d, dtype, oracle):
    """Beyond the fixtures: on fresh tie-free clouds the C restatement and the
    reference's own CPU code (where built) give the same layout and the same
    query answers bit for bit, at several depths and k."""
    if not oracle.ref_available():
        pytest.skip("reference sources are not built here")
    rng = np.random.default_rng(500 + 10 * d + (dtype == np.float64))
    ref = (rng.standard_normal((3000, d)) * 1e3).astype(dtype)
    q = (rng.standard_normal((400, d)) * 1e3).astype(dtype)
    for levels, k in ((1, 3), (4, 9), (7, 17)):
        mine = oracle.build_tree(ref, levels)
        theirs = oracle.RefTree(ref, levels)
        lay = theirs.layout()
        np.testing.assert_array_equal(mine.structured, lay.structured)
        np.testing.assert_array_equal(mine.perm, lay.perm)
        np.testing.assert_array_equal(mine.medians, lay.medians)
        d1, i1 = oracle.query_tree(mine, q, k)
        d2, i2 = theirs.query(q, k)
        np.testing.assert_array_equal(d1, d2)
        np.testing.assert_array_equal(i1, i2)
