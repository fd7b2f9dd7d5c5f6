"""The CPU oracle, pinned to the reference: known-answer tests restated from the reference's
unit tests and the golden outputs the reference itself produced (tests/golden)."""
import numpy as np
import pytest

import oracle
from tests.conftest import kat_graph_arrays, load_golden, sample8_arrays
from tests.golden.cases import cases_for

DOWN, UP = 1, 2


@pytest.fixture(scope="module", autouse=True)
def _build():
    oracle.build()


def test_kat_dot_product_good():
    # test/unit/test_grg.cpp:41-89 (DotProductGood): mutations on nodes 1, 5, 6
    g = oracle.OracleGraph(**kat_graph_arrays((1, 5, 6)))
    out = oracle.matmul(g, np.array([[1.0, 2.0, 1.0]]), DOWN)
    assert out.tolist() == [[1.0, 2.0, 3.0, 3.0]]
    out = oracle.matmul(g, np.ones((1, 4)), UP)
    assert out.tolist() == [[1.0, 2.0, 4.0]]


def test_kat_matrix_mult_good():
    # test/unit/test_grg.cpp:91-124 (MatrixMultGood)
    g = oracle.OracleGraph(**kat_graph_arrays((1, 5, 6)))
    V = np.array([[1.0, 2.0, 1.0], [0.0, 1.0, 1.0]])
    assert oracle.matmul(g, V, DOWN).ravel().tolist() == [1, 2, 3, 3, 1, 1, 2, 2]
    V = np.ones((2, 4))
    V[1] /= 4.0
    np.testing.assert_allclose(oracle.matmul(g, V, UP).ravel(), [1, 2, 4, 0.25, 0.5, 1.0], atol=1e-3)


def test_kat_matmul_bad():
    # test/unit/test_grg.cpp:126-161 (MatMulBad): wrong sizes are API misuse
    g = oracle.OracleGraph(**kat_graph_arrays((1, 5)))
    with pytest.raises(RuntimeError, match="Input vector is not size M"):
        oracle.matmul(g, np.zeros((1, 4)), DOWN)
    with pytest.raises(RuntimeError, match="Input vector is not size N"):
        oracle.matmul(g, np.zeros((1, 3)), UP)
    with pytest.raises(RuntimeError, match="Input vector is not size N"):
        oracle.matmul(g, np.zeros((9, 1)), UP)


def test_kat_xtx():
    # test/unit/test_grg.cpp:258-292 (MatmulXTX): coals(pn4)=coals(pn5)=1, coals(pn6)=0
    a = kat_graph_arrays((6, 5, 4))
    g = oracle.OracleGraph(**a)
    with pytest.raises(RuntimeError, match="Coalescent counts not available"):
        oracle.matmul(g, np.ones((1, 4), dtype=np.int64), UP, init="xtx")
    g = oracle.OracleGraph(**a, coals=np.array([1, 1, 0], dtype=np.uint32))
    assert oracle.matmul(g, np.ones((1, 4), dtype=np.int64), UP, init="xtx").tolist() == [[8, 4, 4]]


def test_kat_change_samples_unordered():
    # test/unit/test_grg.cpp:333-439 (ChangeSamples): {11,41,37,73} UP -> {162,110,52}, also when the
    # node ids are not topologically ordered (pn6 renumbered below its children).
    g = oracle.OracleGraph(**kat_graph_arrays((6, 5, 4)))
    V = np.array([[11, 41, 37, 73]], dtype=np.int64)
    assert oracle.matmul(g, V, UP).tolist() == [[162, 110, 52]]
    # permute: node 4 <-> node 6 (now a parent has a smaller id than its children)
    off = np.array([0, 0, 0, 0, 0, 2, 4, 6], dtype=np.uint64)
    adj = np.array([6, 5, 2, 3, 0, 1], dtype=np.uint32)
    g2 = oracle.OracleGraph(num_samples=4, ploidy=2, down_off=off, down_adj=adj,
                            mut_node=np.array([4, 5, 6], dtype=np.uint32))
    assert oracle.matmul(g2, V, UP).tolist() == [[162, 110, 52]]


def test_kat_sample8_dense():
    # sample8Grg (common_grgs.h:29-57): UP with the identity gives the path-count matrix X
    g = oracle.OracleGraph(**sample8_arrays())
    X = g.dense_X()
    expect = {8: {0, 1}, 9: {0, 1, 2}, 10: {3, 4, 7}, 11: {0, 1, 3, 4, 6, 7}, 12: {3, 4, 5, 7},
              13: {0, 1, 2, 3, 4, 5, 7}}
    for m, node in enumerate(range(8, 14)):
        assert set(np.flatnonzero(X[:, m]).tolist()) == expect[node]
    # DOWN with the identity gives X^T
    assert np.array_equal(oracle.matmul(g, np.eye(6, dtype=np.int64), DOWN), X.T)


@pytest.mark.parametrize("fixture", ["t200", "t200miss", "wt_n1000_m10000"])
def test_oracle_matches_reference_golden(fixture):
    """The restatement reproduces the reference's outputs bit for bit (same summation order)."""
    from tests.conftest import GOLDEN

    z, meta = load_golden(fixture)
    g = oracle.read_grg(GOLDEN / f"{fixture}.grg")
    cases = dict(cases_for(g.num_samples, g.num_mutations, g.num_nodes, g.ploidy, has_miss=bool(meta.get("miss")),
                           profile=meta["profile"]))
    assert sorted(cases) == sorted(meta["cases"])
    for name, (V, direction, kw) in cases.items():
        kw = dict(kw)
        miss = kw.pop("miss", None)
        if miss is not None:
            miss = miss.copy()
        out = oracle.matmul(g, V, direction, miss=miss, **kw)
        assert out.dtype == z[name].dtype and np.array_equal(out, z[name]), name
        if miss is not None and direction == UP:
            assert np.array_equal(miss, z[name + "__miss"]), name


def test_golden_freq_pin():
    """t200's UP int32 ones output is the reference's golden allele count file (checked when the
    fixture was generated from test/endtoend/expect/test-200-samples.freq.txt)."""
    z, meta = load_golden("t200")
    assert meta["freq_pinned"] is True
    counts = z["up_i32_ones_k1"][0]
    assert counts.shape == (10893,) and counts.sum() == 546910


def test_sharded_oracle_matches_plain():
    from tests.conftest import GOLDEN

    g = oracle.read_grg(GOLDEN / "wt_n1000_m10000.grg")
    rng = np.random.default_rng(3)
    sh = oracle.Shards(g, 4)
    for direction, cols in ((UP, g.num_samples), (DOWN, g.num_mutations)):
        V = rng.integers(-50, 50, size=(3, cols)).astype(np.int32)
        assert np.array_equal(sh.matmul(V, direction), oracle.matmul(g, V, direction))


def test_sharded_oracle_ranges_and_alignment():
    """Window-aligned ranged shards: every edge belongs to exactly one shard, a run over a range of
    shards equals the sum (DOWN) / the columns (UP) of its shards, and the whole set equals the
    plain product."""
    g = oracle.window_tree(300, 2500, seed=4, threads=3)
    sh = oracle.Shards(g, 7, build_threads=3, align=100)
    assert sh.edges() == g.num_edges
    rng = np.random.default_rng(6)
    V = rng.integers(-9, 9, size=(2, g.num_mutations)).astype(np.int64)
    parts = [sh.matmul(V, DOWN, first=i, count=1) for i in range(7)]
    assert np.array_equal(sum(parts), oracle.matmul(g, V, DOWN))
    assert np.array_equal(sh.matmul(V, DOWN, first=2, count=3), parts[2] + parts[3] + parts[4])
    U = rng.integers(-9, 9, size=(2, g.num_samples)).astype(np.int32)
    assert np.array_equal(sh.matmul(U, UP), oracle.matmul(g, U, UP))


@pytest.mark.parametrize("N,M,seed", [(2, 5, 1), (777, 1234, 5), (1000, 10000, 42)])
def test_oracle_generator_equals_product_generator(N, M, seed):
    """The oracle's own window-tree generator (window_tree.c) and the product's build the same
    graph bit for bit; the CPU reference arm of the benchmark relies on it."""
    gx = pytest.importorskip("grgl_gb300")
    og = oracle.window_tree(N, M, seed=seed, threads=2)
    a = gx.window_tree_grg(N, M, seed=seed).export_arrays()
    assert np.array_equal(og.down_off, a["down_off"])
    assert np.array_equal(og.down_adj, a["down_adj"])
    assert np.array_equal(og.mut_node, a["mut_node"])


def test_oracle_generator_matches_golden_window_tree():
    """The N=1,000 / M=10,000 seed-42 window-tree genotypes (the golden fixture was built from them
    by the reference constructor): same allele counts from both graphs."""
    from tests.conftest import GOLDEN

    og = oracle.window_tree(1000, 10000, seed=42)
    ref = oracle.read_grg(GOLDEN / "wt_n1000_m10000.grg")
    ones = np.ones((1, 1000), dtype=np.int64)
    assert np.array_equal(oracle.matmul(og, ones, UP), oracle.matmul(ref, ones, UP))


def test_read_grg_missing_nodes():
    from tests.conftest import GOLDEN

    g = oracle.read_grg(GOLDEN / "t200miss.grg")
    assert g.miss_node is not None
    assert np.count_nonzero(g.miss_node != oracle.INVALID_NODE) > 0
